// Device math shared by the setup and operator kernels.
//
// Expansions use the real form of pi-BEM's complex solid-harmonic coefficients
// (include/multipole_expansion.h:102-105): K = (p+1)^2 reals per expansion,
// for each degree n the real part of m = 0 followed by (re, im) of m = 1..n.
// Multipole coefficients are scaled by the box side h (M^_n = M_n / h^n) and
// local coefficients by h^(n+1) (L^_n = L_n h^(n+1)).
#pragma once

#include <cuda_runtime.h>

#include <cmath>

namespace pibem
{
  // (n, m, part) of real index k.
  __host__ __device__ inline void real_index(int k, int &n, int &m, int &part)
  {
    n = 0;
    while ((n + 1) * (n + 1) <= k)
      ++n;
    int r = k - n * n;
    if (r == 0)
      {
        m    = 0;
        part = 0;
      }
    else
      {
        m    = (r + 1) / 2;
        part = (r + 1) % 2; // r odd -> re, even -> im
      }
  }

  // Normalised associated Legendre function P~_n^m(x) = sqrt((n-m)!/(n+m)!) P_n^m(x),
  // Condon-Shortley phase (the normalisation of source/ass_leg_function.cc), by the
  // three-term recurrence; s = sqrt(1-x^2).
  template <typename T>
  __host__ __device__ inline T legendre_nm(int n, int m, T x, T s)
  {
    if (m > n || m < 0)
      return T(0);
    T pmm = T(1);
    for (int i = 1; i <= m; ++i)
      pmm *= -sqrt(T(2 * i - 1) / T(2 * i)) * s;
    if (n == m)
      return pmm;
    T p1 = x * sqrt(T(2 * m + 1)) * pmm;
    T p0 = pmm;
    for (int nn = m + 2; nn <= n; ++nn)
      {
        T p2 = (T(2 * nn - 1) * x * p1 - sqrt(T((nn - 1) * (nn - 1) - m * m)) * p0) /
               sqrt(T(nn * nn - m * m));
        p0 = p1;
        p1 = p2;
      }
    return p1;
  }

  // sqrt(1-x^2) dP~_n^m/dx = -dP~_n^m/dtheta.
  template <typename T>
  __host__ __device__ inline T legendre_dsin(int n, int m, T x, T s)
  {
    T dth;
    if (m == 0)
      dth = n > 0 ? sqrt(T(n) * T(n + 1)) * legendre_nm<T>(n, 1, x, s) : T(0);
    else
      dth = T(0.5) * (sqrt(T(n - m) * T(n + m + 1)) * legendre_nm<T>(n, m + 1, x, s) -
                      sqrt(T(n + m) * T(n - m + 1)) * legendre_nm<T>(n, m - 1, x, s));
    return -dth;
  }

  // Coefficients of the normalised Legendre recurrences for n, m <= 20:
  //   P~_m^m     = -cmm[m] s P~_{m-1}^{m-1},       cmm[m] = sqrt((2m-1)/(2m))
  //   P~_{m+1}^m = cm1[m] x P~_m^m,                cm1[m] = sqrt(2m+1)
  //   P~_n^m     = ra[n][m] x P~_{n-1}^m - rb[n][m] P~_{n-2}^m,
  //                ra = (2n-1)/sqrt(n^2-m^2), rb = sqrt((n-1)^2-m^2)/sqrt(n^2-m^2)
  struct LegendreTables
  {
    double cmm[21], cm1[21], ra[21][21], rb[21][21];
    float  fcmm[21], fcm1[21], fra[21][21], frb[21][21];
    float2 ffcmm[21], ffcm1[21], ffra[21][21], ffrb[21][21]; // (hi, lo) pairs
  };
  // One copy per translation unit that evaluates expansions; filled by
  // fill_legendre_tables() + cudaMemcpyToSymbol from that unit.
  static __constant__ LegendreTables c_leg;

  inline void fill_legendre_tables(LegendreTables &t)
  {
    auto pair = [](double v) {
      const float hi = float(v);
      return make_float2(hi, float(v - double(hi)));
    };
    for (int m = 0; m <= 20; ++m)
      {
        t.cmm[m] = m > 0 ? std::sqrt((2.0 * m - 1.0) / (2.0 * m)) : 0.0;
        t.cm1[m] = std::sqrt(2.0 * m + 1.0);
        for (int n = 0; n <= 20; ++n)
          {
            bool ok    = n >= m + 2;
            t.ra[n][m] = ok ? (2.0 * n - 1.0) / std::sqrt(double(n * n - m * m)) : 0.0;
            t.rb[n][m] = ok ? std::sqrt(double((n - 1) * (n - 1) - m * m)) / std::sqrt(double(n * n - m * m)) : 0.0;
            t.fra[n][m] = float(t.ra[n][m]);
            t.frb[n][m] = float(t.rb[n][m]);
            t.ffra[n][m] = pair(t.ra[n][m]);
            t.ffrb[n][m] = pair(t.rb[n][m]);
          }
        t.fcmm[m] = float(t.cmm[m]);
        t.fcm1[m] = float(t.cm1[m]);
        t.ffcmm[m] = pair(t.cmm[m]);
        t.ffcm1[m] = pair(t.cm1[m]);
      }
  }

  template <typename T>
  struct LegT;
  template <>
  struct LegT<double>
  {
    __device__ static double cmm(int m) { return c_leg.cmm[m]; }
    __device__ static double cm1(int m) { return c_leg.cm1[m]; }
    __device__ static double ra(int n, int m) { return c_leg.ra[n][m]; }
    __device__ static double rb(int n, int m) { return c_leg.rb[n][m]; }
  };
  template <>
  struct LegT<float>
  {
    __device__ static float cmm(int m) { return c_leg.fcmm[m]; }
    __device__ static float cm1(int m) { return c_leg.fcm1[m]; }
    __device__ static float ra(int n, int m) { return c_leg.fra[n][m]; }
    __device__ static float rb(int n, int m) { return c_leg.frb[n][m]; }
  };

  // Table-driven evaluation (same sum as eval_expansion below, no square roots
  // in the loop): value = sum_k coef[k] basis_k(r).
  template <typename T, typename E>
  __device__ inline T eval_expansion_fast(const E *__restrict__ coef, int p, T rx, T ry, T rz,
                                          bool multipole)
  {
    using LT = LegT<T>;
    const T r2  = rx * rx + ry * ry + rz * rz;
    const T rho = sqrt(r2);
    const T inv = T(1) / rho;
    const T x   = rz * inv;
    const T s   = sqrt(fmax(T(0), T(1) - x * x));
    const T rxy = sqrt(rx * rx + ry * ry);
    T       cb = T(1), sb = T(0);
    if (rxy > T(0))
      {
        cb = rx / rxy;
        sb = ry / rxy;
      }
    const T step = multipole ? inv : rho;
    T       acc  = T(0);
    T       pmm  = T(1);
    T       rpm  = multipole ? inv : T(1);
    T       cm = T(1), sm = T(0);
    for (int m = 0; m <= p; ++m)
      {
        if (m > 0)
          {
            pmm *= -LT::cmm(m) * s;
            rpm *= step;
            const T c2 = cm * cb - sm * sb;
            sm         = sm * cb + cm * sb;
            cm         = c2;
          }
        const T cr = m == 0 ? T(1) : T(2) * cm;
        const T ci = m == 0 ? T(0) : -T(2) * sm;
        T       p0 = pmm, rp = rpm;
        int     k0 = m * m + (m == 0 ? 0 : 2 * m - 1);
        T       v  = T(coef[k0]) * cr + (m > 0 ? T(coef[k0 + 1]) * ci : T(0));
        acc += v * p0 * rp;
        if (m + 1 <= p)
          {
            T p1 = x * LT::cm1(m) * pmm;
            rp *= step;
            int n  = m + 1;
            k0     = n * n + (m == 0 ? 0 : 2 * m - 1);
            v      = T(coef[k0]) * cr + (m > 0 ? T(coef[k0 + 1]) * ci : T(0));
            acc += v * p1 * rp;
            for (n = m + 2; n <= p; ++n)
              {
                const T p2 = LT::ra(n, m) * x * p1 - LT::rb(n, m) * p0;
                p0         = p1;
                p1         = p2;
                rp *= step;
                k0 = n * n + (m == 0 ? 0 : 2 * m - 1);
                v  = T(coef[k0]) * cr + (m > 0 ? T(coef[k0 + 1]) * ci : T(0));
                acc += v * p1 * rp;
              }
          }
      }
    return acc;
  }

  // Evaluation of a scaled expansion at relative position r (in box units):
  //   kind 0 (local):     sum_k E[k] * basis_k with r^n
  //   kind 1 (multipole): with r^(-n-1)
  // value = Re sum_n [E_n^0 P~ r^. + 2 sum_m E_n^m e^{im beta} P~ r^.]
  // (MultipoleExpansion::Evaluate multipole_expansion.cc:265-298,
  //  LocalExpansion::Evaluate local_expansion.cc:252-287).
  // Runs the recurrence m-major so that the whole sum costs O(K).
  template <typename T, typename E>
  __device__ inline T eval_expansion(const E *coef, int p, T rx, T ry, T rz, bool multipole)
  {
    T rho = sqrt(rx * rx + ry * ry + rz * rz);
    T x   = rz / rho;
    T s   = sqrt(fmax(T(0), T(1) - x * x));
    T rxy = sqrt(rx * rx + ry * ry);
    T cb = T(1), sb = T(0);
    if (rxy > T(0))
      {
        cb = rx / rxy;
        sb = ry / rxy;
      }
    T base = multipole ? T(1) / rho : T(1); // rho^(-1) or rho^0 at n = m = 0
    T step = multipole ? T(1) / rho : rho;
    T acc  = T(0);
    T pmm  = T(1);
    T rpm  = base;       // rho power at n = m
    T cm = T(1), sm = T(0); // cos(m beta), sin(m beta)
    for (int m = 0; m <= p; ++m)
      {
        if (m > 0)
          {
            pmm *= -sqrt(T(2 * m - 1) / T(2 * m)) * s;
            rpm *= step;
            T c2 = cm * cb - sm * sb;
            sm   = sm * cb + cm * sb;
            cm   = c2;
          }
        // n = m
        T p0 = pmm, rp = rpm;
        T cr = m == 0 ? T(1) : T(2) * cm, ci = m == 0 ? T(0) : -T(2) * sm;
        auto term = [&](int n, T P, T r) {
          int k0 = n * n + (m == 0 ? 0 : 2 * m - 1);
          T   v  = T(coef[k0]) * cr;
          if (m > 0)
            v += T(coef[k0 + 1]) * ci;
          acc += v * P * r;
        };
        term(m, p0, rp);
        if (m + 1 <= p)
          {
            T p1 = x * sqrt(T(2 * m + 1)) * pmm;
            T r1 = rp * step;
            term(m + 1, p1, r1);
            for (int n = m + 2; n <= p; ++n)
              {
                T p2 = (T(2 * n - 1) * x * p1 - sqrt(T((n - 1) * (n - 1) - m * m)) * p0) /
                       sqrt(T(n * n - m * m));
                p0 = p1;
                p1 = p2;
                r1 *= step;
                term(n, p1, r1);
              }
          }
      }
    return acc;
  }
} // namespace pibem
