// Oracle: CPU restatement of pi-BEM's FMM collocation BEM operator
// (source/bem_fma.cc), its dense collocation operator (source/bem_problem.cc
// ONE_BODY assemble_system) and the solve around them (source/bem_problem.cc
// compute_alpha / vmult / compute_rhs / solve_system).
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle against which the GPU
// implementation is compared; the product never links, loads or calls it.
//
// The data structures deliberately mirror the reference (std::set interaction
// lists, per-block maps of cell -> quadrature-point ids, complex expansions in
// the reference's triangular storage) so that each step can be read next to
// the reference file:line it restates.  Third-party pieces the reference takes
// from deal.II (QGauss, QTelles, bilinear FE_Q(1) geometry, GMRES) are restated
// from their published definitions; see the comments at each.
#include "pibem_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <vector>

namespace
{
  using cplx = std::complex<double>;
  constexpr double PI   = 3.14159265358979323846;
  constexpr double TOLL = 0.001; // source/bem_fma.cc:1

  inline int tri(int n, int m) { return n * (n + 1) / 2 + m; } // multipole_expansion.h:102-105
  inline int ncoef(int p) { return (p + 1) * (p + 2) / 2; }

  // ------------------------------------------------------------------
  // Associated Legendre functions, reference normalisation
  // P~_n^m = sqrt((n-m)!/(n+m)!) P_n^m with the Condon-Shortley phase
  // (source/ass_leg_function.cc closed forms, e.g. P_1_1 = -sqrt(2)/2 sqrt(1-x^2)).
  // Restated with the standard three-term recurrence in normalised form.
  // ------------------------------------------------------------------
  struct Legendre
  {
    int                 nmax;
    std::vector<double> P;  // tri(n,m)
    std::vector<double> dS; // sqrt(1-x^2) * dP~/dx = -dP~/dtheta
    void eval(int nmax_, double x, bool deriv)
    {
      nmax = nmax_;
      P.assign(ncoef(nmax), 0.0);
      const double s = std::sqrt(std::max(0.0, 1.0 - x * x));
      P[0]           = 1.0;
      for (int m = 1; m <= nmax; ++m)
        P[tri(m, m)] = -std::sqrt((2.0 * m - 1.0) / (2.0 * m)) * s * P[tri(m - 1, m - 1)];
      for (int m = 0; m < nmax; ++m)
        P[tri(m + 1, m)] = x * std::sqrt(2.0 * m + 1.0) * P[tri(m, m)];
      for (int m = 0; m <= nmax; ++m)
        for (int n = m + 2; n <= nmax; ++n)
          P[tri(n, m)] = ((2.0 * n - 1.0) * x * P[tri(n - 1, m)] -
                          std::sqrt(double((n - 1) * (n - 1) - m * m)) * P[tri(n - 2, m)]) /
                         std::sqrt(double(n * n - m * m));
      if (!deriv)
        return;
      dS.assign(ncoef(nmax), 0.0);
      for (int n = 0; n <= nmax; ++n)
        for (int m = 0; m <= n; ++m)
          {
            double dth;
            if (m == 0)
              dth = n > 0 ? std::sqrt(double(n) * (n + 1)) * P[tri(n, 1)] : 0.0;
            else
              {
                double up = m < n ? std::sqrt(double(n - m) * (n + m + 1)) * P[tri(n, m + 1)] : 0.0;
                double dn = std::sqrt(double(n + m) * (n - m + 1)) * P[tri(n, m - 1)];
                dth       = 0.5 * (up - dn);
              }
            dS[tri(n, m)] = -dth;
          }
    }
  };

  // A_n^m = (-1)^n / sqrt((n-m)!(n+m)!), multipole_expansion.h:124-147.
  struct AnmTable
  {
    double a[21][21];
    AnmTable()
    {
      for (int n = 0; n <= 20; ++n)
        for (int m = 0; m <= n; ++m)
          {
            double f1 = 1., f2 = 1.;
            for (int ii = n - m; ii > 0; ii--)
              f1 *= ii;
            for (int ii = n + m; ii > 0; ii--)
              f2 *= ii;
            a[n][m] = std::pow(-1., double(n)) / std::sqrt(f1 * f2);
          }
    }
    double operator()(int n, int m) const { return a[n][std::abs(m)]; }
  };
  const AnmTable &Anm()
  {
    static AnmTable t;
    return t;
  }
  // Re(i^k) for the even exponents that occur in the translation factors.
  inline double re_ipow(int k)
  {
    int r = ((k % 4) + 4) % 4;
    return r == 0 ? 1.0 : (r == 2 ? -1.0 : 0.0);
  }
  inline int sgn(int x) { return x < 0 ? -1 : (x > 0 ? 1 : 0); }

  struct P3
  {
    double x, y, z;
  };
  inline void spherical(const P3 &r, double &rho, double &cosa, double &beta)
  {
    rho  = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    cosa = r.z / rho;
    beta = std::atan2(r.y, r.x);
  }

  // ------------------------------------------------------------------
  // Complex expansions (reference storage and formulas).
  // ------------------------------------------------------------------
  struct Expansion
  {
    int               p = 0;
    P3                c{0, 0, 0};
    std::vector<cplx> a;
    bool              is_zero = true;
    Expansion() {}
    Expansion(int p_, P3 c_) : p(p_), c(c_), a(ncoef(p_), cplx(0, 0)) {}
  };

  // MultipoleExpansion::Add(strength, point), multipole_expansion.cc:94-122.
  void p2m_point(Expansion &M, double q, const P3 &x)
  {
    if (q == 0)
      return;
    M.is_zero = false;
    double rho, ca, be;
    spherical(P3{x.x - M.c.x, x.y - M.c.y, x.z - M.c.z}, rho, ca, be);
    Legendre L;
    L.eval(M.p, ca, false);
    for (int n = 0; n <= M.p; ++n)
      for (int m = 0; m <= n; ++m)
        {
          double rf = L.P[tri(n, m)] * std::pow(rho, double(n)) * q;
          M.a[tri(n, m)] += std::polar(1.0, -m * be) * rf;
        }
  }

  // MultipoleExpansion::AddNormDer, multipole_expansion.cc:125-181.
  void p2m_dipole(Expansion &M, double q, const P3 &x, const P3 &nrm)
  {
    if (q == 0)
      return;
    M.is_zero      = false;
    P3     r{x.x - M.c.x, x.y - M.c.y, x.z - M.c.z};
    double nn      = std::sqrt(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
    P3     nv{nrm.x / nn, nrm.y / nn, nrm.z / nn};
    double rho     = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    double dRhodN  = (r.x / rho) * nv.x + (r.y / rho) * nv.y + (r.z / rho) * nv.z;
    double beta    = std::atan2(r.y, r.x);
    double rxy2    = r.x * r.x + r.y * r.y;
    double dBetadN = (-r.y / rxy2) * nv.x + (r.x / rxy2) * nv.y;
    double ca      = r.z / rho;
    double sa      = std::sqrt(std::max(0.0, 1. - ca * ca));
    double dAlphadN =
      (ca * std::cos(beta) / rho) * nv.x + (ca * std::sin(beta) / rho) * nv.y + (-sa / rho) * nv.z;
    Legendre L;
    L.eval(M.p, ca, true);
    for (int n = 0; n <= M.p; ++n)
      for (int m = 0; m <= n; ++m)
        {
          double P  = L.P[tri(n, m)];
          double dP = L.dS[tri(n, m)];
          double rn = std::pow(rho, double(n));
          cplx   z  = std::polar(1.0, -double(m) * beta);
          z *= cplx(double(n) * std::pow(rho, double(n) - 1.) * P * dRhodN - rn * dP * dAlphadN,
                    -double(m) * rn * P * dBetadN);
          z *= q;
          M.a[tri(n, m)] += z;
        }
  }

  // MultipoleExpansion::Add(M, s), multipole_expansion.cc:75-91.
  void add_scaled(Expansion &dst, const Expansion &src, double s)
  {
    if (src.is_zero || s == 0)
      return;
    dst.is_zero = false;
    for (size_t i = 0; i < dst.a.size(); ++i)
      dst.a[i] += src.a[i] * s;
  }

  // MultipoleExpansion::Add(child) (M2M), multipole_expansion.cc:185-261.
  void m2m(Expansion &par, const Expansion &ch)
  {
    if (ch.is_zero)
      return;
    par.is_zero = false;
    P3     r{ch.c.x - par.c.x, ch.c.y - par.c.y, ch.c.z - par.c.z};
    double d = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    if (!(d > 1e-7))
      {
        for (size_t i = 0; i < par.a.size(); ++i)
          par.a[i] += ch.a[i];
        return;
      }
    double rho, ca, be;
    spherical(r, rho, ca, be);
    Legendre L;
    L.eval(par.p, ca, false);
    const AnmTable &A = Anm();
    const int       p = par.p;
    for (int n = 0; n <= p; ++n)
      for (int m = 0; m <= n; ++m)
        {
          cplx z(0, 0);
          for (int nn = 0; nn <= n; ++nn)
            for (int mm = -nn; mm <= nn; ++mm)
              {
                if (std::abs(m - mm) > n - nn)
                  continue;
                const cplx &o = ch.a[tri(n - nn, std::abs(m - mm))];
                cplx        av(o.real(), sgn(m - mm) * o.imag());
                double      rf = L.P[tri(nn, std::abs(mm))] * std::pow(rho, double(nn)) * A(nn, mm) *
                            A(n - nn, m - mm) / A(n, m);
                rf *= re_ipow(std::abs(m) - std::abs(mm) - std::abs(m - mm));
                z += rf * (av * std::polar(1.0, -mm * be));
              }
          par.a[tri(n, m)] += z;
        }
  }

  // LocalExpansion::Add(M) (M2L), local_expansion.cc:180-248 with the factor
  // table of local_expansion.h:146-180.
  void m2l(Expansion &loc, const Expansion &M)
  {
    if (M.is_zero)
      return;
    P3     r{M.c.x - loc.c.x, M.c.y - loc.c.y, M.c.z - loc.c.z};
    double rho, ca, be;
    spherical(r, rho, ca, be);
    const int p = loc.p;
    Legendre  L;
    L.eval(2 * p, ca, false);
    const AnmTable   &A = Anm();
    std::vector<cplx> e(4 * p + 1);
    for (int k = -2 * p; k <= 2 * p; ++k)
      e[k + 2 * p] = cplx(std::cos(k * be), std::sin(k * be));
    for (int n = 0; n <= p; ++n)
      for (int m = 0; m <= n; ++m)
        {
          cplx z(0, 0);
          for (int nn = 0; nn <= p; ++nn)
            {
              double rhoFact = std::pow(rho, double(-n - nn - 1));
              for (int mm = -nn; mm <= nn; ++mm)
                {
                  cplx a = M.a[tri(nn, std::abs(mm))];
                  if (mm < 0)
                    a = std::conj(a);
                  double C = A(nn, mm) / A(n + nn, m - mm) * A(n, m) *
                             re_ipow(std::abs(m - mm) - std::abs(m) - std::abs(mm)) /
                             std::pow(-1., nn);
                  double rf = L.P[tri(nn + n, std::abs(mm - m))] * rhoFact * C;
                  z += a * e[mm - m + 2 * p] * rf;
                }
            }
          loc.a[tri(n, m)] += z;
        }
    loc.is_zero = false;
  }

  // LocalExpansion::Add(L) (L2L), local_expansion.cc:108-176 with the factor
  // table of local_expansion.h:183-215.
  void l2l(Expansion &ch, const Expansion &par)
  {
    if (par.is_zero)
      return;
    const int p = ch.p;
    P3        r{par.c.x - ch.c.x, par.c.y - ch.c.y, par.c.z - ch.c.z};
    double    d = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    if (!(d > 1e-7))
      {
        for (size_t i = 0; i < ch.a.size(); ++i)
          ch.a[i] += par.a[i];
        ch.is_zero = false;
        return;
      }
    double rho, ca, be;
    spherical(r, rho, ca, be);
    Legendre L;
    L.eval(p, ca, false);
    const AnmTable &A = Anm();
    for (int n = 0; n <= p; ++n)
      for (int m = 0; m <= n; ++m)
        {
          cplx z(0, 0);
          for (int nn = n; nn <= p; ++nn)
            {
              double rhoFact = std::pow(rho, double(nn - n));
              for (int mm = -nn; mm <= nn; ++mm)
                {
                  if (std::abs(mm - m) > nn - n)
                    continue;
                  const cplx &o = par.a[tri(nn, std::abs(mm))];
                  cplx        a(o.real(), sgn(mm) * o.imag());
                  double      LC = A(nn - n, mm - m) / A(nn, mm) * A(n, m) *
                              re_ipow(std::abs(mm) - std::abs(mm - m) - std::abs(m)) *
                              std::pow(-1., nn + n);
                  double rf = L.P[tri(nn - n, std::abs(mm - m))] * rhoFact * LC;
                  z += a * cplx(std::cos((mm - m) * be), std::sin((mm - m) * be)) * rf;
                }
            }
          ch.a[tri(n, m)] += z;
        }
    ch.is_zero = false;
  }

  // MultipoleExpansion::Evaluate (M2P), multipole_expansion.cc:265-298.
  double m2p(const Expansion &M, const P3 &x)
  {
    if (M.is_zero)
      return 0.0;
    double rho, ca, be;
    spherical(P3{x.x - M.c.x, x.y - M.c.y, x.z - M.c.z}, rho, ca, be);
    Legendre L;
    L.eval(M.p, ca, false);
    cplx f(0, 0);
    for (int n = 0; n <= M.p; ++n)
      {
        double rf = std::pow(rho, double(-n - 1));
        f += M.a[tri(n, 0)] * (L.P[tri(n, 0)] * rf);
        for (int m = 1; m <= n; ++m)
          f += M.a[tri(n, m)] * std::polar(1.0, m * be) * 2. * (L.P[tri(n, m)] * rf);
      }
    return f.real();
  }

  // LocalExpansion::Evaluate (L2P), local_expansion.cc:252-287.
  double l2p(const Expansion &Lx, const P3 &x)
  {
    if (Lx.is_zero)
      return 0.0;
    double rho, ca, be;
    spherical(P3{x.x - Lx.c.x, x.y - Lx.c.y, x.z - Lx.c.z}, rho, ca, be);
    Legendre L;
    L.eval(Lx.p, ca, false);
    cplx f(0, 0);
    for (int n = 0; n <= Lx.p; ++n)
      {
        double rf = std::pow(rho, double(n));
        f += Lx.a[tri(n, 0)] * (L.P[tri(n, 0)] * rf);
        for (int m = 1; m <= n; ++m)
          f += Lx.a[tri(n, m)] * (cplx(std::cos(m * be), std::sin(m * be)) * 2. * (L.P[tri(n, m)] * rf));
      }
    return f.real();
  }

  // ------------------------------------------------------------------
  // Quadrature rules on [0,1] (restated from their published definitions).
  // ------------------------------------------------------------------
  // Gauss-Legendre n-point rule by Newton iteration on P_n (Golub-Welsch
  // equivalent); points ascending on [0,1], weights summing to 1.
  void gauss01(int n, std::vector<double> &x, std::vector<double> &w)
  {
    x.assign(n, 0);
    w.assign(n, 0);
    for (int i = 0; i < n; ++i)
      {
        double z = std::cos(PI * (i + 0.75) / (n + 0.5));
        double pp = 0;
        for (int it = 0; it < 100; ++it)
          {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j)
              {
                double p3 = p2;
                p2        = p1;
                p1        = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
              }
            pp        = n * (z * p1 - p2) / (z * z - 1.0);
            double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16)
              break;
          }
        {
          double p1 = 1, p2 = 0;
          for (int j = 1; j <= n; ++j)
            {
              double p3 = p2;
              p2        = p1;
              p1        = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
          pp = n * (z * p1 - p2) / (z * z - 1.0);
        }
        // z descends with i; store ascending on [0,1]
        x[n - 1 - i] = 0.5 * (1.0 - z) ;
        w[n - 1 - i] = 1.0 / ((1.0 - z * z) * pp * pp);
      }
    // x currently holds (1-z)/2 for descending z -> ascending already; fix ordering
    std::vector<std::pair<double, double>> xw(n);
    for (int i = 0; i < n; ++i)
      xw[i] = {x[i], w[i]};
    std::sort(xw.begin(), xw.end());
    for (int i = 0; i < n; ++i)
      {
        x[i] = xw[i].first;
        w[i] = xw[i].second;
      }
  }

  // Telles (1987) cubic transformation of an n-point Gauss rule, clustering at
  // the end s in {0,1} of [0,1]: eta_bar = 2s-1, eta* = eta_bar^2-1 = 0, hence
  // gamma_bar = eta_bar;  eta(g) = ((g-gb)^3 + gb(gb^2+3))/(1+3gb^2),
  // d eta/d g = 3(g-gb)^2/(1+3gb^2).
  void telles01(int n, int s, std::vector<double> &x, std::vector<double> &w)
  {
    std::vector<double> gx, gw;
    gauss01(n, gx, gw);
    double eb = 2.0 * s - 1.0, es = eb * eb - 1.0;
    double gb = (es == 0.0) ? eb
                            : std::cbrt(eb * es + std::fabs(es)) + std::cbrt(eb * es - std::fabs(es)) + eb;
    x.resize(n);
    w.resize(n);
    for (int q = 0; q < n; ++q)
      {
        double g   = gx[q] * 2 - 1;
        double eta = (std::pow(g - gb, 3.0) + gb * (gb * gb + 3)) / (1 + 3 * gb * gb);
        double J   = 3 * ((g - gb) * (g - gb)) / (1 + 3 * gb * gb);
        x[q]       = (eta + 1) / 2.0;
        w[q]       = gw[q] * J;
      }
  }

  // 2-D tensor rules, x index fastest (deal.II tensor-product ordering).
  void rule2d(const std::vector<double> &x1, const std::vector<double> &w1,
              const std::vector<double> &x2, const std::vector<double> &w2,
              std::vector<double> &pts, std::vector<double> &w)
  {
    pts.clear();
    w.clear();
    for (size_t j = 0; j < x2.size(); ++j)
      for (size_t i = 0; i < x1.size(); ++i)
        {
          pts.push_back(x1[i]);
          pts.push_back(x2[j]);
          w.push_back(w1[i] * w2[j]);
        }
  }

  // Bilinear (FE_Q(1) / MappingQ1) geometry of a quadrilateral cell at unit
  // coordinates (xi, eta); vertices in deal.II lexicographic order.  The
  // position is formed without fused multiply-adds in a fixed order so that
  // the GPU code, which uses the same order, produces identical points.
  struct CellGeo
  {
    P3     x, n;
    double J;
    double N[4];
  };
  void cell_geo(const P3 *v, double xi, double eta, CellGeo &g)
  {
    volatile double a0 = (1 - xi) * (1 - eta), a1 = xi * (1 - eta), a2 = (1 - xi) * eta,
                    a3 = xi * eta;
    g.N[0] = a0;
    g.N[1] = a1;
    g.N[2] = a2;
    g.N[3] = a3;
    auto comb = [&](double c0, double c1, double c2, double c3) {
      volatile double t0 = c0 * a0;
      volatile double t1 = c1 * a1;
      volatile double s  = t0 + t1;
      volatile double t2 = c2 * a2;
      s                  = s + t2;
      volatile double t3 = c3 * a3;
      s                  = s + t3;
      return (double)s;
    };
    g.x.x = comb(v[0].x, v[1].x, v[2].x, v[3].x);
    g.x.y = comb(v[0].y, v[1].y, v[2].y, v[3].y);
    g.x.z = comb(v[0].z, v[1].z, v[2].z, v[3].z);
    P3 tx{(1 - eta) * (v[1].x - v[0].x) + eta * (v[3].x - v[2].x),
          (1 - eta) * (v[1].y - v[0].y) + eta * (v[3].y - v[2].y),
          (1 - eta) * (v[1].z - v[0].z) + eta * (v[3].z - v[2].z)};
    P3 ty{(1 - xi) * (v[2].x - v[0].x) + xi * (v[3].x - v[1].x),
          (1 - xi) * (v[2].y - v[0].y) + xi * (v[3].y - v[1].y),
          (1 - xi) * (v[2].z - v[0].z) + xi * (v[3].z - v[1].z)};
    P3 c{tx.y * ty.z - tx.z * ty.y, tx.z * ty.x - tx.x * ty.z, tx.x * ty.y - tx.y * ty.x};
    g.J = std::sqrt(c.x * c.x + c.y * c.y + c.z * c.z);
    g.n = P3{c.x / g.J, c.y / g.J, c.z / g.J};
  }

  // LaplaceKernel::kernels (include/laplace_kernel.h:55-74):
  // s = 1/(4 pi r), D = R / (-4 pi r^3), R = q - x_i.
  inline void kernels(const P3 &R, P3 &D, double &s)
  {
    double r  = std::sqrt(R.x * R.x + R.y * R.y + R.z * R.z);
    double r2 = r * r;
    s         = 1. / (r * 4 * PI);
    double f  = -4 * PI * r2 * r;
    D         = P3{R.x / f, R.y / f, R.z / f};
  }

  // ------------------------------------------------------------------
  // Octree block (include/octree_block.h:70-97).
  // ------------------------------------------------------------------
  struct Block
  {
    int                            level = 0, parent = 0, nchild = 0;
    int                            child[8];
    double                         pmin[3];
    double                         delta = 0;
    std::vector<int>               nodes;
    std::map<int, std::vector<int>> quads; // cell -> quad point ids
    std::vector<std::set<int>>     nn, il, nil;
    Block() : nn(1), il(1), nil(1) {}
  };

  struct Row
  {
    std::vector<int>    cols;
    std::vector<double> N, D;
  };
} // namespace

struct orc_handle
{
  int p, L, max_nodes, qorder, sorder, external;
  // mesh
  int                            n_nodes = 0, n_cells = 0;
  std::vector<P3>                xyz;
  std::vector<int>               cells; // 4 per cell
  std::vector<std::set<int>>     dbl;
  std::vector<std::vector<int>>  dof_to_elems;
  int                            nq = 0; // quad points per cell
  std::vector<P3>                qpts, qnrm;
  std::vector<double>            qjxw, qshape; // qshape[(c*nq+q)*4+j]
  std::vector<unsigned char>     dir;
  bool                           have_dirichlet = true;
  // octree
  std::vector<Block>             blocks;
  std::vector<int>               startLevel, endLevel, childless;
  std::vector<std::vector<int>>  dofs_filled;
  std::vector<std::vector<std::vector<int>>> qp_to_block; // [cell][q] -> block per level
  // near field (CSR rows)
  std::vector<Row>               near;
  // P2M element tables: per childless block: map cell -> 4 expansions each kernel
  std::vector<std::map<int, std::vector<Expansion>>> elemM1, elemM2;
  // expansions of the last matvec
  std::vector<Expansion>         M1, M2, L1, L2;
  // dense
  std::vector<double>            denseN, denseD;
  // double body: the dense matrices add the mesh reflected in z = z0
  int                            double_body = 0;
  double                         z0 = 0.0;
  // constraint lines of the solve: x[row] - (col >= 0 ? x[col] : 0) = g
  std::vector<int>               con_row, con_col;
  std::vector<double>            con_g;
  // preconditioner of orc_solve: 0 none, 1 leaf-block Jacobi (right), 2 ILU(0)
  // of the near-field system matrix (BEMFMA::FMA_preconditioner)
  int                            prec = 0;
  std::vector<std::vector<double>> blk_inv; // per childless block, row-major m x m
  std::vector<int64_t>           ilu_ptr;   // CSR of the ILU(0) factors (L unit lower, U)
  std::vector<int>               ilu_col, ilu_diag;
  std::vector<double>            ilu_val;
  // Telles rules per singular vertex, Gauss rule
  std::vector<double>            gpts, gw;
  std::vector<double>            tpts[4], tw[4];

  P3 center(int b) const
  {
    const Block &B = blocks[b];
    return P3{B.pmin[0] + B.delta / 2., B.pmin[1] + B.delta / 2., B.pmin[2] + B.delta / 2.};
  }
};

namespace
{
  // Regular / singular integration of one cell for collocation node i over the
  // quadrature-point subset qs (regular) or the whole cell with Telles
  // clustering at vertex sv (singular) -- bem_fma.cc:670-913, 997-1153.
  void integrate_cell(const orc_handle *h, int i, int c, const std::vector<int> *qs, int sv,
                      double Nr[4], double Dr[4])
  {
    for (int j = 0; j < 4; ++j)
      Nr[j] = Dr[j] = 0;
    const P3 &xi = h->xyz[i];
    if (sv < 0)
      {
        for (int q : *qs)
          {
            size_t k = size_t(c) * h->nq + q;
            P3     R{h->qpts[k].x - xi.x, h->qpts[k].y - xi.y, h->qpts[k].z - xi.z};
            P3     D;
            double s;
            kernels(R, D, s);
            double dn = D.x * h->qnrm[k].x + D.y * h->qnrm[k].y + D.z * h->qnrm[k].z;
            for (int j = 0; j < 4; ++j)
              {
                Nr[j] += (dn * h->qshape[k * 4 + j] * h->qjxw[k]);
                Dr[j] += (s * h->qshape[k * 4 + j] * h->qjxw[k]);
              }
          }
      }
    else
      {
        P3 v[4];
        for (int j = 0; j < 4; ++j)
          v[j] = h->xyz[h->cells[4 * c + j]];
        const std::vector<double> &tp = h->tpts[sv], &tw = h->tw[sv];
        for (size_t q = 0; q < tw.size(); ++q)
          {
            CellGeo g;
            cell_geo(v, tp[2 * q], tp[2 * q + 1], g);
            P3     R{g.x.x - xi.x, g.x.y - xi.y, g.x.z - xi.z};
            P3     D;
            double s;
            kernels(R, D, s);
            double dn  = D.x * g.n.x + D.y * g.n.y + D.z * g.n.z;
            double jxw = g.J * tw[q];
            for (int j = 0; j < 4; ++j)
              {
                Nr[j] += (dn * g.N[j] * jxw);
                Dr[j] += (s * g.N[j] * jxw);
              }
          }
      }
  }

  int singular_vertex(const orc_handle *h, int i, int c)
  {
    for (int j = 0; j < 4; ++j)
      if (h->dbl[i].count(h->cells[4 * c + j]))
        return j;
    return -1;
  }

  // Touch test of bem_fma.cc:4323-4360 (absolute tolerance TOLL).
  bool touches(const Block &b1, const Block &b2)
  {
    double PMin1[3], PMax1[3], PMin2[3], PMax2[3];
    for (int k = 0; k < 3; ++k)
      {
        PMin1[k] = b1.pmin[k];
        PMax1[k] = 2. * (b1.delta / 2.) + b1.pmin[k];
        PMin2[k] = b2.pmin[k];
        PMax2[k] = 2. * (b2.delta / 2.) + b2.pmin[k];
      }
    for (int a = 0; a < 3; ++a)
      {
        int o1 = (a + 1) % 3, o2 = (a + 2) % 3;
        if ((std::fabs(PMin1[a] - PMax2[a]) <= TOLL) || (std::fabs(PMax1[a] - PMin2[a]) <= TOLL))
          if ((PMin1[o1] - TOLL <= PMax2[o1]) && (PMax1[o1] + TOLL >= PMin2[o1]))
            if ((PMin1[o2] - TOLL <= PMax2[o2]) && (PMax1[o2] + TOLL >= PMin2[o2]))
              return true;
      }
    return false;
  }

  // Child index of a point inside a parent box, bem_fma.cc:3844-3973:
  // 0:(0,0,0) 1:(1,0,0) 2:(1,1,0) 3:(0,1,0) 4:(0,0,1) 5:(1,0,1) 6:(1,1,1) 7:(0,1,1);
  // a coordinate on the split plane goes to the low side.
  int child_index(const P3 &x, const double pmin[3], double delta)
  {
    bool hz = !(x.z <= pmin[2] + delta);
    bool hy = !(x.y <= pmin[1] + delta);
    bool hx = !(x.x <= pmin[0] + delta);
    static const int tab[2][2][2] = {{{0, 1}, {3, 2}}, {{4, 5}, {7, 6}}};
    return tab[hz][hy][hx];
  }
  const int child_off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

  // BEMFMA::generate_octree_blocking, bem_fma.cc:3615-4801.
  void build_tree(orc_handle *h)
  {
    const int L = h->L;
    double    max_coor = 0;
    for (auto &x : h->xyz)
      max_coor = std::max({max_coor, std::fabs(x.x), std::fabs(x.y), std::fabs(x.z)});
    h->blocks.clear();
    h->startLevel.assign(L + 1, 0);
    h->endLevel.assign(L + 1, 0);
    h->childless.clear();
    h->dofs_filled.assign(L + 1, {});
    std::vector<std::vector<int>> parentList(L + 1);
    parentList[0].push_back(0);
    h->qp_to_block.assign(h->n_cells, std::vector<std::vector<int>>(h->nq));

    Block root;
    root.level  = 0;
    root.parent = 0;
    for (int k = 0; k < 3; ++k)
      root.pmin[k] = -1.1 * max_coor;
    double delta = 2.2 * max_coor;
    root.delta   = delta;
    for (int c = 0; c < h->n_cells; ++c)
      for (int q = 0; q < h->nq; ++q)
        {
          root.quads[c].push_back(q);
          h->qp_to_block[c][q].push_back(0);
        }
    for (int i = 0; i < h->n_nodes; ++i)
      root.nodes.push_back(i);
    h->blocks.push_back(root);

    for (int level = 1; level <= L; ++level)
      {
        delta /= 2.;
        for (int jj : parentList[level - 1])
          {
            Block ch[8];
            double pm[3] = {h->blocks[jj].pmin[0], h->blocks[jj].pmin[1], h->blocks[jj].pmin[2]};
            for (int j = 0; j < 8; ++j)
              {
                ch[j].level  = level;
                ch[j].parent = jj;
                ch[j].delta  = delta;
                for (int k = 0; k < 3; ++k)
                  ch[j].pmin[k] = pm[k] + (child_off[j][k] ? delta : 0.);
              }
            for (int i : h->blocks[jj].nodes)
              ch[child_index(h->xyz[i], pm, delta)].nodes.push_back(i);
            for (auto &kv : h->blocks[jj].quads)
              for (int q : kv.second)
                ch[child_index(h->qpts[size_t(kv.first) * h->nq + q], pm, delta)]
                  .quads[kv.first]
                  .push_back(q);
            for (int j = 0; j < 8; ++j)
              if (ch[j].nodes.size() + ch[j].quads.size() > 0)
                {
                  int id = int(h->blocks.size());
                  h->blocks.push_back(ch[j]);
                  Block &P = h->blocks[jj];
                  P.child[P.nchild++] = id;
                  for (auto &kv : h->blocks[id].quads)
                    for (int q : kv.second)
                      h->qp_to_block[kv.first][q].push_back(id);
                }
          }
        h->startLevel[level] = h->endLevel[level - 1] + 1;
        h->endLevel[level]   = int(h->blocks.size()) - 1;
        for (int jj = h->startLevel[level]; jj <= h->endLevel[level]; ++jj)
          {
            Block &B          = h->blocks[jj];
            double numNodes   = 0.0;
            for (int i : B.nodes)
              numNodes += 1.0 / double(h->dbl[i].size());
            if (std::round(numNodes) <= h->max_nodes)
              {
                h->childless.push_back(jj);
                for (auto &kv : B.quads)
                  for (int q : kv.second)
                    for (int j = level + 1; j <= L; ++j)
                      h->qp_to_block[kv.first][q].push_back(jj);
              }
            else
              parentList[level].push_back(jj);
            if (numNodes > 0)
              h->dofs_filled[level].push_back(jj);
          }
      }
    for (int jj : parentList[L])
      h->childless.push_back(jj);

    // Near neighbours, bem_fma.cc:4269-4580.
    auto &blocks = h->blocks;
    if (L >= 1)
      for (int ii = h->startLevel[1]; ii <= h->endLevel[1]; ++ii)
        for (int jj = h->startLevel[1]; jj <= h->endLevel[1]; ++jj)
          blocks[ii].nn[0].insert(jj);
    for (int level = 2; level <= L; ++level)
      for (int kk = h->startLevel[level]; kk <= h->endLevel[level]; ++kk)
        {
          Block &b1 = blocks[kk];
          b1.nn[0].insert(kk);
          for (int pos : blocks[b1.parent].nn[0])
            {
              if (blocks[pos].nchild == 0 && touches(b1, blocks[pos]))
                b1.nn[0].insert(pos);
              for (int c = 0; c < blocks[pos].nchild; ++c)
                if (touches(b1, blocks[blocks[pos].child[c]]))
                  b1.nn[0].insert(blocks[pos].child[c]);
            }
          if (b1.nchild == 0)
            {
              int ns = L - level + 1;
              b1.nn.resize(ns);
              b1.il.resize(ns);
              b1.nil.resize(ns);
              for (int sub = 1; sub < ns; ++sub)
                for (int pos : std::set<int>(b1.nn[sub - 1]))
                  {
                    if (blocks[pos].nchild == 0)
                      b1.nn[sub].insert(pos);
                    for (int c = 0; c < blocks[pos].nchild; ++c)
                      if (touches(b1, blocks[blocks[pos].child[c]]))
                        b1.nn[sub].insert(blocks[pos].child[c]);
                  }
            }
        }

    // Interaction and non-interaction lists, bem_fma.cc:4588-4711.
    if (L >= 1)
      for (int ii = h->startLevel[1]; ii <= h->endLevel[1]; ++ii)
        for (int jj = h->startLevel[1]; jj <= h->endLevel[1]; ++jj)
          blocks[ii].il[0].insert(jj);
    for (int level = 2; level <= L; ++level)
      for (int jj = h->startLevel[level]; jj <= h->endLevel[level]; ++jj)
        {
          Block &b1 = blocks[jj];
          for (size_t sub = 0; sub < b1.nn.size(); ++sub)
            {
              b1.il[sub].insert(b1.nn[sub].begin(), b1.nn[sub].end());
              for (int node : b1.nodes)
                for (int d : h->dbl[node])
                  for (int c : h->dof_to_elems[d])
                    for (int q = 0; q < h->nq; ++q)
                      b1.il[sub].insert(h->qp_to_block[c][q][level + sub]);
            }
          for (size_t sub = 0; sub < b1.nn.size(); ++sub)
            {
              const std::set<int> &il = b1.il[sub];
              const std::set<int> &pil =
                (sub == 0) ? blocks[b1.parent].il[0] : b1.il[sub - 1];
              for (int pos : pil)
                {
                  const Block &b2 = blocks[pos];
                  if (b2.nchild == 0)
                    {
                      if (!il.count(pos))
                        b1.nil[sub].insert(pos);
                    }
                  else
                    for (int c = 0; c < b2.nchild; ++c)
                      if (!il.count(b2.child[c]))
                        b1.nil[sub].insert(b2.child[c]);
                }
            }
        }
  }

  // BEMFMA::direct_integrals, bem_fma.cc:108-1600.  Rows are assembled per
  // collocation node: first the childless-block (intList) part, then for
  // level = 1..L the coarser non-interaction blocks of the node's block at that
  // level -- the order of the reference's copier calls.
  void build_near(orc_handle *h)
  {
    auto &blocks = h->blocks;
    int   nb     = int(blocks.size());
    // cell -> quad subset maps per block
    std::vector<std::map<int, std::set<int>>> il_map(nb), coarse_map(nb);
    std::vector<char>                         has_coarse(nb, 0);
    for (int b : h->childless)
      {
        const Block &B = blocks[b];
        if (B.nodes.empty())
          continue;
        for (int pos : B.il[B.il.size() - 1])
          for (auto &kv : blocks[pos].quads)
            il_map[b][kv.first].insert(kv.second.begin(), kv.second.end());
      }
    for (int level = 1; level <= h->L; ++level)
      for (int b : h->dofs_filled[level])
        {
          const Block &B = blocks[b];
          for (size_t sub = 0; sub < B.nn.size(); ++sub)
            for (int pos : B.nil[sub])
              {
                if (pos >= h->startLevel[level])
                  break;
                for (auto &kv : blocks[pos].quads)
                  coarse_map[b][kv.first].insert(kv.second.begin(), kv.second.end());
              }
          has_coarse[b] = 1;
        }
    // block of each node at each level
    std::vector<std::vector<int>> node_block(h->n_nodes, std::vector<int>(h->L + 1, -1));
    std::vector<int>              node_leaf(h->n_nodes, -1);
    for (int b = 0; b < nb; ++b)
      for (int i : blocks[b].nodes)
        node_block[i][blocks[b].level] = b;
    for (int b : h->childless)
      for (int i : blocks[b].nodes)
        node_leaf[i] = b;

    h->near.assign(h->n_nodes, Row());
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < h->n_nodes; ++i)
      {
        std::map<int, std::pair<double, double>> row;
        auto add_entries = [&](const std::map<int, std::set<int>> &m, bool allow_singular) {
          for (auto &kv : m)
            {
              int                c  = kv.first;
              std::vector<int>   qs(kv.second.begin(), kv.second.end());
              int                sv = allow_singular ? singular_vertex(h, i, c) : -1;
              double             Nr[4], Dr[4];
              integrate_cell(h, i, c, &qs, sv, Nr, Dr);
              for (int j = 0; j < 4; ++j)
                {
                  auto &e = row[h->cells[4 * c + j]];
                  e.first += Nr[j];
                  e.second += Dr[j];
                }
            }
        };
        int lb = node_leaf[i];
        if (lb >= 0)
          add_entries(il_map[lb], true);
        for (int level = 1; level <= h->L; ++level)
          {
            int b = node_block[i][level];
            if (b >= 0 && has_coarse[b])
              add_entries(coarse_map[b], false);
          }
        Row &r = h->near[i];
        for (auto &kv : row)
          {
            r.cols.push_back(kv.first);
            r.N.push_back(kv.second.first);
            r.D.push_back(kv.second.second);
          }
      }
  }

  // BEMFMA::multipole_integrals, bem_fma.cc:1609-1840.
  void build_p2m(orc_handle *h)
  {
    int nc = int(h->childless.size());
    h->elemM1.assign(h->blocks.size(), {});
    h->elemM2.assign(h->blocks.size(), {});
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < nc; ++k)
      {
        int          b  = h->childless[k];
        const Block &B  = h->blocks[b];
        P3           cb = h->center(b);
        for (auto &kv : B.quads)
          {
            int                    c = kv.first;
            std::vector<Expansion> e1(4, Expansion(h->p, cb)), e2(4, Expansion(h->p, cb));
            for (int q : kv.second)
              {
                size_t kq = size_t(c) * h->nq + q;
                for (int j = 0; j < 4; ++j)
                  {
                    double s = h->qshape[kq * 4 + j] * h->qjxw[kq] / 4 / PI;
                    p2m_dipole(e1[j], s, h->qpts[kq], h->qnrm[kq]);
                    p2m_point(e2[j], s, h->qpts[kq]);
                  }
              }
            h->elemM1[b][c] = e1;
            h->elemM2[b][c] = e2;
          }
      }
  }

  void fmm_matvec(orc_handle *h, const double *phi, const double *dphi, double *outN,
                  double *outD)
  {
    const int nb = int(h->blocks.size());
    // near field SpMV, bem_fma.cc:2408-2409
#pragma omp parallel for schedule(static)
    for (int i = 0; i < h->n_nodes; ++i)
      {
        const Row &r = h->near[i];
        double     sn = 0, sd = 0;
        for (size_t k = 0; k < r.cols.size(); ++k)
          {
            sn += r.N[k] * phi[r.cols[k]];
            sd += r.D[k] * dphi[r.cols[k]];
          }
        outN[i] = sn;
        outD[i] = sd;
      }
    // generate_multipole_expansions, bem_fma.cc:1971-2380
    h->M1.assign(nb, Expansion());
    h->M2.assign(nb, Expansion());
    for (int b = 0; b < nb; ++b)
      {
        h->M1[b] = Expansion(h->p, h->center(b));
        h->M2[b] = Expansion(h->p, h->center(b));
      }
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < int(h->childless.size()); ++k)
      {
        int b = h->childless[k];
        for (auto &kv : h->blocks[b].quads)
          {
            int c = kv.first;
            for (int j = 0; j < 4; ++j)
              {
                int d = h->cells[4 * c + j];
                add_scaled(h->M2[b], h->elemM2[b].at(c)[j], dphi[d]);
                add_scaled(h->M1[b], h->elemM1[b].at(c)[j], phi[d]);
              }
          }
      }
    for (int level = h->L; level > 0; --level)
      {
        if (h->endLevel[level] < h->startLevel[level])
          continue;
        // parents of this level, each summing its children in ascending order
        std::vector<int> parents;
        for (int kk = h->startLevel[level]; kk <= h->endLevel[level]; ++kk)
          if (parents.empty() || parents.back() != h->blocks[kk].parent)
            parents.push_back(h->blocks[kk].parent);
#pragma omp parallel for schedule(dynamic, 4)
        for (int pi = 0; pi < int(parents.size()); ++pi)
          {
            int          par = parents[pi];
            const Block &P   = h->blocks[par];
            for (int c = 0; c < P.nchild; ++c)
              {
                int kk = P.child[c];
                for (int ker = 0; ker < 2; ++ker)
                  {
                    std::vector<Expansion> &M = ker ? h->M2 : h->M1;
                    Expansion               t(h->p, M[par].c);
                    m2m(t, M[kk]);
                    m2m(M[par], t);
                  }
              }
          }
      }
    // multipole_matr_vect_products, bem_fma.cc:2391-3072
    h->L1.assign(nb, Expansion());
    h->L2.assign(nb, Expansion());
    for (int b = 0; b < nb; ++b)
      {
        h->L1[b] = Expansion(h->p, h->center(b));
        h->L2[b] = Expansion(h->p, h->center(b));
      }
    for (int level = 1; level <= h->L; ++level)
      {
        if (h->endLevel[level] < h->startLevel[level])
          continue;
        const int sL = h->startLevel[level], eL = h->endLevel[level];
        const std::vector<int> &fl = h->dofs_filled[level];
#pragma omp parallel for schedule(dynamic, 4)
        for (int t = 0; t < int(fl.size()); ++t)
          {
            int          kk = fl[t];
            const Block &B  = h->blocks[kk];
            Expansion    l1(h->p, h->center(kk)), l2(h->p, h->center(kk));
            l2l(l1, h->L1[B.parent]);
            l2l(l2, h->L2[B.parent]);
            std::vector<double> cN(B.nodes.size(), 0.0), cD(B.nodes.size(), 0.0);
            for (size_t sub = 0; sub < B.nn.size(); ++sub)
              for (int pos : B.nil[sub])
                {
                  if (pos < sL)
                    continue;
                  if (pos <= eL)
                    {
                      m2l(l1, h->M1[pos]);
                      m2l(l2, h->M2[pos]);
                    }
                  else
                    for (size_t ii = 0; ii < B.nodes.size(); ++ii)
                      {
                        const P3 &x = h->xyz[B.nodes[ii]];
                        cN[ii] += m2p(h->M1[pos], x);
                        cD[ii] += m2p(h->M2[pos], x);
                      }
                }
            l2l(h->L1[kk], l1);
            l2l(h->L2[kk], l2);
            for (size_t ii = 0; ii < B.nodes.size(); ++ii)
              {
                outD[B.nodes[ii]] += cD[ii];
                outN[B.nodes[ii]] += cN[ii];
              }
          }
      }
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < int(h->childless.size()); ++k)
      {
        int b = h->childless[k];
        for (int i : h->blocks[b].nodes)
          {
            outD[i] += l2p(h->L2[b], h->xyz[i]);
            outN[i] += l2p(h->L1[b], h->xyz[i]);
          }
      }
  }

  // The reflected cell of BEMProblem::_assemble_system_double_body
  // (bem_problem.cc:1036-1062 for a regular pair, :1100-1121 for a singular
  // one: the same regular rule either way): the quadrature points mirrored in
  // z = z0, the normal's z component negated, the cell's own shape values and
  // JxW.  The row's cell part is added by the caller.
  void integrate_reflected_cell(const orc_handle *h, int i, int c, double Nr[4], double Dr[4])
  {
    for (int j = 0; j < 4; ++j)
      Nr[j] = Dr[j] = 0;
    const P3 &xi = h->xyz[i];
    for (int q = 0; q < h->nq; ++q)
      {
        size_t k = size_t(c) * h->nq + q;
        P3     R{h->qpts[k].x - xi.x, h->qpts[k].y - xi.y, 2.0 * h->z0 - h->qpts[k].z - xi.z};
        P3     nr{h->qnrm[k].x, h->qnrm[k].y, -h->qnrm[k].z};
        P3     D;
        double s;
        kernels(R, D, s);
        double dn = D.x * nr.x + D.y * nr.y + D.z * nr.z;
        for (int j = 0; j < 4; ++j)
          {
            Nr[j] += (dn * h->qshape[k * 4 + j] * h->qjxw[k]);
            Dr[j] += (s * h->qshape[k * 4 + j] * h->qjxw[k]);
          }
      }
  }

  // Dense one-body collocation matrices (bem_problem.cc:478-950, without the
  // matrix print), with the same regular and singular rules as the FMM near
  // field.
  void build_dense(orc_handle *h)
  {
    size_t n = h->n_nodes;
    h->denseN.assign(n * n, 0.0);
    h->denseD.assign(n * n, 0.0);
    std::vector<int> all(h->nq);
    for (int q = 0; q < h->nq; ++q)
      all[q] = q;
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < h->n_nodes; ++i)
      for (int c = 0; c < h->n_cells; ++c)
        {
          double Nr[4], Dr[4];
          integrate_cell(h, i, c, &all, singular_vertex(h, i, c), Nr, Dr);
          if (h->double_body)
            {
              double Nm[4], Dm[4];
              integrate_reflected_cell(h, i, c, Nm, Dm);
              for (int j = 0; j < 4; ++j)
                {
                  Nr[j] += Nm[j];
                  Dr[j] += Dm[j];
                }
            }
          for (int j = 0; j < 4; ++j)
            {
              h->denseN[size_t(i) * n + h->cells[4 * c + j]] += Nr[j];
              h->denseD[size_t(i) * n + h->cells[4 * c + j]] += Dr[j];
            }
        }
  }

  void dense_matvec(orc_handle *h, const double *phi, const double *dphi, double *outN,
                    double *outD)
  {
    if (h->denseN.empty())
      build_dense(h);
    size_t n = h->n_nodes;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < h->n_nodes; ++i)
      {
        double sn = 0, sd = 0;
        for (size_t j = 0; j < n; ++j)
          {
            sn += h->denseN[i * n + j] * phi[j];
            sd += h->denseD[i * n + j] * dphi[j];
          }
        outN[i] = sn;
        outD[i] = sd;
      }
  }

  void op_matvec(orc_handle *h, int dense, const double *a, const double *b, double *oN,
                 double *oD)
  {
    if (dense)
      dense_matvec(h, a, b, oN, oD);
    else
      fmm_matvec(h, a, b, oN, oD);
  }

  double norm2(const std::vector<double> &v)
  {
    double s = 0;
    for (double x : v)
      s += x * x;
    return std::sqrt(s);
  }
} // namespace

extern "C"
{
  orc_handle *orc_create(int p, int L, int max_nodes, int qorder, int sorder, int external)
  {
    orc_handle *h = new orc_handle();
    h->p          = p;
    h->L          = L;
    h->max_nodes  = max_nodes;
    h->qorder     = qorder;
    h->sorder     = sorder;
    h->external   = external;
    std::vector<double> g, w;
    gauss01(qorder, g, w);
    rule2d(g, w, g, w, h->gpts, h->gw);
    for (int v = 0; v < 4; ++v)
      {
        std::vector<double> tx, twx, ty, twy;
        telles01(sorder, v & 1, tx, twx);
        telles01(sorder, (v >> 1) & 1, ty, twy);
        rule2d(tx, twx, ty, twy, h->tpts[v], h->tw[v]);
      }
    return h;
  }

  void orc_destroy(orc_handle *h) { delete h; }
  void orc_set_threads(int n) { omp_set_num_threads(n); }

  int orc_set_mesh(orc_handle *h, int n_nodes, const double *xyz, int n_cells, const int *cells,
                   const int *doff, const int *dids)
  {
    h->n_nodes = n_nodes;
    h->n_cells = n_cells;
    h->xyz.resize(n_nodes);
    for (int i = 0; i < n_nodes; ++i)
      h->xyz[i] = P3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    h->cells.assign(cells, cells + 4 * size_t(n_cells));
    h->dbl.assign(n_nodes, {});
    for (int i = 0; i < n_nodes; ++i)
      {
        if (doff)
          for (int k = doff[i]; k < doff[i + 1]; ++k)
            h->dbl[i].insert(dids[k]);
        h->dbl[i].insert(i);
      }
    h->dof_to_elems.assign(n_nodes, {});
    for (int c = 0; c < n_cells; ++c)
      for (int j = 0; j < 4; ++j)
        h->dof_to_elems[cells[4 * c + j]].push_back(c);
    h->nq = int(h->gw.size());
    size_t nqt = size_t(n_cells) * h->nq;
    h->qpts.resize(nqt);
    h->qnrm.resize(nqt);
    h->qjxw.resize(nqt);
    h->qshape.resize(nqt * 4);
    for (int c = 0; c < n_cells; ++c)
      {
        P3 v[4];
        for (int j = 0; j < 4; ++j)
          v[j] = h->xyz[cells[4 * c + j]];
        for (int q = 0; q < h->nq; ++q)
          {
            CellGeo g;
            cell_geo(v, h->gpts[2 * q], h->gpts[2 * q + 1], g);
            size_t k    = size_t(c) * h->nq + q;
            h->qpts[k]  = g.x;
            h->qnrm[k]  = g.n;
            h->qjxw[k]  = g.J * h->gw[q];
            for (int j = 0; j < 4; ++j)
              h->qshape[k * 4 + j] = g.N[j];
          }
      }
    h->dir.assign(n_nodes, 1);
    h->denseN.clear();
    h->denseD.clear();
    build_tree(h);
    build_near(h);
    build_p2m(h);
    return 0;
  }

  int orc_set_double_body(orc_handle *h, int on, double z0)
  {
    h->double_body = on ? 1 : 0;
    h->z0          = z0;
    h->denseN.clear();
    h->denseD.clear();
    return 0;
  }

  int orc_set_bc(orc_handle *h, const unsigned char *mask)
  {
    h->dir.assign(mask, mask + h->n_nodes);
    h->have_dirichlet = false;
    for (int i = 0; i < h->n_nodes; ++i)
      if (h->dir[i])
        h->have_dirichlet = true;
    return 0;
  }

  void orc_fmm_matvec(orc_handle *h, const double *phi, const double *dphi, double *oN,
                      double *oD)
  {
    fmm_matvec(h, phi, dphi, oN, oD);
  }
  void orc_dense_matvec(orc_handle *h, const double *phi, const double *dphi, double *oN,
                        double *oD)
  {
    dense_matvec(h, phi, dphi, oN, oD);
  }

  // BEMProblem::compute_alpha, bem_problem.cc:1139-1162: alpha = -N*1 for
  // interior flow; -1 - N*1 for exterior flow (the double-layer jump on the
  // other side of the surface).
  void orc_compute_alpha(orc_handle *h, int dense, double *alpha)
  {
    size_t              n = h->n_nodes;
    std::vector<double> ones(n, -1.0), zeros(n, 0.0), dummy(n);
    op_matvec(h, dense, ones.data(), zeros.data(), alpha, dummy.data());
    if (h->external)
      for (size_t i = 0; i < n; ++i)
        alpha[i] -= 1.0;
  }

  // BEMProblem::vmult, bem_problem.cc:1165-1217.
  void orc_system_matvec(orc_handle *h, int dense, const double *alpha, const double *x, double *y)
  {
    size_t              n = h->n_nodes;
    std::vector<double> sphi(x, x + n), sdphi(x, x + n), oN(n), oD(n);
    if (!h->have_dirichlet)
      {
        double nr = norm2(sphi);
        for (auto &v : sphi)
          v -= nr;
      }
    for (size_t i = 0; i < n; ++i)
      {
        sphi[i] *= h->dir[i] ? 0.0 : 1.0;
        sdphi[i] *= h->dir[i] ? 1.0 : 0.0;
      }
    op_matvec(h, dense, sphi.data(), sdphi.data(), oN.data(), oD.data());
    for (size_t i = 0; i < n; ++i)
      y[i] = -oD[i] + oN[i] + alpha[i] * sphi[i];
    if (!h->have_dirichlet)
      {
        std::vector<double> t(y, y + n);
        double              nr = norm2(t);
        for (size_t i = 0; i < n; ++i)
          y[i] -= nr;
      }
  }

  // BEMProblem::compute_rhs, bem_problem.cc:1220-1260.
  void orc_compute_rhs(orc_handle *h, int dense, const double *alpha, const double *tmp,
                       double *rhs)
  {
    size_t              n = h->n_nodes;
    std::vector<double> sphi(n), sdphi(n), oN(n), oD(n);
    for (size_t i = 0; i < n; ++i)
      {
        sphi[i]  = h->dir[i] ? tmp[i] : 0.0;
        sdphi[i] = h->dir[i] ? 0.0 : tmp[i];
      }
    op_matvec(h, dense, sphi.data(), sdphi.data(), oN.data(), oD.data());
    for (size_t i = 0; i < n; ++i)
      rhs[i] = -(oN[i] + alpha[i] * sphi[i]) + oD[i];
  }

  // BEMProblem::solve_system, bem_problem.cc:1267-1347, with an own restarted
  // GMRES (modified Gram-Schmidt, Givens rotations) on the true residual.
  // ConstrainedOperator::vmult (include/constrained_matrix.h:100-125): the
  // system operator, then every constrained row replaced by its constraint
  // x[row] - w x[col].
  static void constrained_matvec(orc_handle *h, int dense, const double *alpha, const double *x,
                                 double *y)
  {
    orc_system_matvec(h, dense, alpha, x, y);
    for (size_t k = 0; k < h->con_row.size(); ++k)
      {
        const int i = h->con_row[k];
        y[i]        = x[i] - (h->con_col[k] >= 0 ? x[h->con_col[k]] : 0.0);
      }
  }

  int orc_set_constraints(orc_handle *h, int n, const int *rows, const int *cols, const double *g)
  {
    h->con_row.assign(rows, rows + n);
    h->con_col.assign(cols, cols + n);
    h->con_g.assign(g, g + n);
    return 0;
  }

  // Leaf-block Jacobi, the GPU library's preconditioner (not the reference's:
  // its FMA branch defines an ILU of the near field, bem_fma.cc:3080-3411, whose
  // use in solve_system is commented out, bem_problem.cc:1300-1304).  Per
  // childless block, the dense inverse of the near-field system matrix
  // (BEMProblem::vmult's near part: N on Neumann columns, -D on Dirichlet
  // columns, alpha on the diagonal of Neumann rows) restricted to the block's
  // own nodes; a constrained row is its constraint line.
  static void build_block_jacobi(orc_handle *h, const double *alpha)
  {
    const int           nc = int(h->childless.size());
    std::vector<int>    con(h->n_nodes, -2); // -2: free row, else the line's column (-1: none)
    for (size_t k = 0; k < h->con_row.size(); ++k)
      con[h->con_row[k]] = h->con_col[k];
    h->blk_inv.assign(nc, {});
#pragma omp parallel for schedule(dynamic, 8)
    for (int kb = 0; kb < nc; ++kb)
      {
        const std::vector<int> &nodes = h->blocks[h->childless[kb]].nodes;
        const int               m     = int(nodes.size());
        std::vector<double>     a(size_t(m) * m, 0.0), inv(size_t(m) * m, 0.0);
        for (int r = 0; r < m; ++r)
          {
            const int i = nodes[r];
            if (con[i] != -2)
              {
                a[size_t(r) * m + r] = 1.0;
                for (int c = 0; c < m; ++c)
                  if (nodes[c] == con[i] && c != r)
                    a[size_t(r) * m + c] -= 1.0;
                continue;
              }
            const Row &row = h->near[i];
            for (int c = 0; c < m; ++c)
              {
                const int j  = nodes[c];
                auto      it = std::lower_bound(row.cols.begin(), row.cols.end(), j);
                if (it != row.cols.end() && *it == j)
                  {
                    size_t e = size_t(it - row.cols.begin());
                    a[size_t(r) * m + c] = h->dir[j] ? -row.D[e] : row.N[e];
                  }
              }
            if (!h->dir[i])
              a[size_t(r) * m + r] += alpha[i];
          }
        // Gauss-Jordan with partial pivoting
        for (int r = 0; r < m; ++r)
          inv[size_t(r) * m + r] = 1.0;
        for (int c = 0; c < m; ++c)
          {
            int piv = c;
            for (int r = c + 1; r < m; ++r)
              if (std::fabs(a[size_t(r) * m + c]) > std::fabs(a[size_t(piv) * m + c]))
                piv = r;
            if (piv != c)
              for (int t = 0; t < m; ++t)
                {
                  std::swap(a[size_t(c) * m + t], a[size_t(piv) * m + t]);
                  std::swap(inv[size_t(c) * m + t], inv[size_t(piv) * m + t]);
                }
            const double d = a[size_t(c) * m + c];
            for (int t = 0; t < m; ++t)
              {
                a[size_t(c) * m + t] /= d;
                inv[size_t(c) * m + t] /= d;
              }
            for (int r = 0; r < m; ++r)
              if (r != c && a[size_t(r) * m + c] != 0.0)
                {
                  const double f = a[size_t(r) * m + c];
                  for (int t = 0; t < m; ++t)
                    {
                      a[size_t(r) * m + t] -= f * a[size_t(c) * m + t];
                      inv[size_t(r) * m + t] -= f * inv[size_t(c) * m + t];
                    }
                }
          }
        h->blk_inv[kb].swap(inv);
      }
  }

  // BEMFMA::FMA_preconditioner (bem_fma.cc:3080-3411): the matrix on the
  // sparsity pattern of the near field (init_prec_sparsity_pattern), N on
  // Neumann and -D on Dirichlet columns (init_preconditioner, :952-962), alpha
  // added on the diagonal of unconstrained Neumann rows (:3293-3308); a
  // constrained row holds 1 on its diagonal and each constraint entry's weight
  // as it is stored (:3190-3201, set(i, entry.first, entry.second): +1 for a
  // double-node line x_d = x_i).  Then TrilinosWrappers::PreconditionILU with
  // its default parameters (:3408): ILU(0), no fill, no diagonal
  // perturbation (Ifpack's classical IKJ factorisation on the matrix pattern).
  static void build_ilu(orc_handle *h, const double *alpha)
  {
    const int        n = h->n_nodes;
    std::vector<int> con(n, -2); // -2: unconstrained, else the line's column (-1: none)
    for (size_t k = 0; k < h->con_row.size(); ++k)
      con[h->con_row[k]] = h->con_col[k];
    h->ilu_ptr.assign(n + 1, 0);
    h->ilu_col.clear();
    h->ilu_val.clear();
    for (int i = 0; i < n; ++i)
      {
        if (con[i] != -2)
          {
            std::vector<std::pair<int, double>> e = {{i, 1.0}};
            if (con[i] >= 0 && con[i] != i)
              e.push_back({con[i], 1.0});
            std::sort(e.begin(), e.end());
            for (auto &p : e)
              {
                h->ilu_col.push_back(p.first);
                h->ilu_val.push_back(p.second);
              }
          }
        else
          {
            const Row &row = h->near[i];
            for (size_t k = 0; k < row.cols.size(); ++k)
              {
                const int j = row.cols[k];
                double    v = h->dir[j] ? -row.D[k] : row.N[k];
                if (j == i && !h->dir[i])
                  v += alpha[i];
                h->ilu_col.push_back(j);
                h->ilu_val.push_back(v);
              }
          }
        h->ilu_ptr[i + 1] = int64_t(h->ilu_col.size());
      }
    h->ilu_diag.assign(n, -1);
    for (int i = 0; i < n; ++i)
      for (int64_t e = h->ilu_ptr[i]; e < h->ilu_ptr[i + 1]; ++e)
        if (h->ilu_col[e] == i)
          h->ilu_diag[i] = int(e);
    // IKJ ILU(0): for each row i, for its columns k < i in ascending order,
    // a_ik /= a_kk, then a_ij -= a_ik a_kj for the columns j > k of row k that
    // row i also holds
    std::vector<int64_t> pos(n, -1);
    for (int i = 0; i < n; ++i)
      {
        for (int64_t e = h->ilu_ptr[i]; e < h->ilu_ptr[i + 1]; ++e)
          pos[h->ilu_col[e]] = e;
        for (int64_t e = h->ilu_ptr[i]; e < h->ilu_ptr[i + 1] && h->ilu_col[e] < i; ++e)
          {
            const int k = h->ilu_col[e];
            h->ilu_val[e] /= h->ilu_val[h->ilu_diag[k]];
            const double lik = h->ilu_val[e];
            for (int64_t f = h->ilu_diag[k] + 1; f < h->ilu_ptr[k + 1]; ++f)
              {
                const int64_t q = pos[h->ilu_col[f]];
                if (q >= 0)
                  h->ilu_val[q] -= lik * h->ilu_val[f];
              }
          }
        for (int64_t e = h->ilu_ptr[i]; e < h->ilu_ptr[i + 1]; ++e)
          pos[h->ilu_col[e]] = -1;
      }
  }

  // z = (L U)^-1 v
  static void apply_ilu(const orc_handle *h, const double *v, double *z)
  {
    const int n = h->n_nodes;
    for (int i = 0; i < n; ++i)
      {
        double s = v[i];
        for (int64_t e = h->ilu_ptr[i]; e < h->ilu_diag[i]; ++e)
          s -= h->ilu_val[e] * z[h->ilu_col[e]];
        z[i] = s;
      }
    for (int i = n - 1; i >= 0; --i)
      {
        double s = z[i];
        for (int64_t e = h->ilu_diag[i] + 1; e < h->ilu_ptr[i + 1]; ++e)
          s -= h->ilu_val[e] * z[h->ilu_col[e]];
        z[i] = s / h->ilu_val[h->ilu_diag[i]];
      }
  }

  static void apply_preconditioner(const orc_handle *h, const double *v, double *z);

  static void apply_block_jacobi(const orc_handle *h, const double *v, double *z)
  {
    const int nc = int(h->childless.size());
#pragma omp parallel for schedule(static)
    for (int kb = 0; kb < nc; ++kb)
      {
        const std::vector<int> &nodes = h->blocks[h->childless[kb]].nodes;
        const int               m     = int(nodes.size());
        const double           *inv   = h->blk_inv[kb].data();
        for (int r = 0; r < m; ++r)
          {
            double s = 0;
            for (int c = 0; c < m; ++c)
              s += inv[size_t(r) * m + c] * v[nodes[c]];
            z[nodes[r]] = s;
          }
      }
  }

  static void apply_preconditioner(const orc_handle *h, const double *v, double *z)
  {
    if (h->prec == 2)
      apply_ilu(h, v, z);
    else
      apply_block_jacobi(h, v, z);
  }

  void orc_set_preconditioner(orc_handle *h, int kind) { h->prec = kind; }

  int64_t orc_preconditioner_build(orc_handle *h, int kind)
  {
    std::vector<double> alpha(h->n_nodes);
    orc_compute_alpha(h, 0, alpha.data());
    h->prec = kind;
    if (kind == 1)
      build_block_jacobi(h, alpha.data());
    else if (kind == 2)
      {
        build_ilu(h, alpha.data());
        return int64_t(h->ilu_col.size());
      }
    return 0;
  }

  void orc_preconditioner_apply(orc_handle *h, const double *v, double *z)
  {
    if (h->prec == 0)
      std::copy(v, v + h->n_nodes, z);
    else
      apply_preconditioner(h, v, z);
  }

  void orc_ilu_factors(orc_handle *h, int64_t *ptr, int32_t *col, double *val)
  {
    std::copy(h->ilu_ptr.begin(), h->ilu_ptr.end(), ptr);
    std::copy(h->ilu_col.begin(), h->ilu_col.end(), col);
    std::copy(h->ilu_val.begin(), h->ilu_val.end(), val);
  }

  int orc_solve(orc_handle *h, int dense, double *phi, double *dphi, const double *tmp, double tol,
                int max_steps, int restart, double *final_res)
  {
    size_t              n = h->n_nodes;
    std::vector<double> alpha(n), b(n), x(n), r(n), w(n);
    orc_compute_alpha(h, dense, alpha.data());
    orc_compute_rhs(h, dense, alpha.data(), tmp, b.data());
    if (h->prec == 1)
      build_block_jacobi(h, alpha.data());
    else if (h->prec == 2)
      build_ilu(h, alpha.data());
    // ConstrainedOperator::distribute_rhs (include/constrained_matrix.h:172-181)
    for (size_t k = 0; k < h->con_row.size(); ++k)
      b[h->con_row[k]] = h->con_g[k];
    x           = b; // initial guess = rhs (bem_problem.cc:1295)
    double bn   = norm2(b);
    int    its  = 0;
    double rel  = 1.0;
    if (bn == 0)
      bn = 1;
    while (its < max_steps)
      {
        constrained_matvec(h, dense, alpha.data(), x.data(), w.data());
        for (size_t i = 0; i < n; ++i)
          r[i] = b[i] - w[i];
        double beta = norm2(r);
        rel         = beta / bn;
        if (rel <= tol)
          break;
        int                              m = restart;
        std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
        std::vector<std::vector<double>> H(m + 1, std::vector<double>(m, 0.0));
        std::vector<double>              cs(m), sn(m), g(m + 1, 0.0), z(n);
        for (size_t i = 0; i < n; ++i)
          V[0][i] = r[i] / beta;
        g[0]  = beta;
        int k = 0;
        for (; k < m && its < max_steps; ++k)
          {
            ++its;
            if (h->prec)
              {
                apply_preconditioner(h, V[k].data(), z.data());
                constrained_matvec(h, dense, alpha.data(), z.data(), w.data());
              }
            else
              constrained_matvec(h, dense, alpha.data(), V[k].data(), w.data());
            for (int i = 0; i <= k; ++i)
              {
                double s = 0;
                for (size_t t = 0; t < n; ++t)
                  s += w[t] * V[i][t];
                H[i][k] = s;
                for (size_t t = 0; t < n; ++t)
                  w[t] -= s * V[i][t];
              }
            H[k + 1][k] = norm2(w);
            for (size_t t = 0; t < n; ++t)
              V[k + 1][t] = w[t] / H[k + 1][k];
            for (int i = 0; i < k; ++i)
              {
                double t1 = cs[i] * H[i][k] + sn[i] * H[i + 1][k];
                H[i + 1][k] = -sn[i] * H[i][k] + cs[i] * H[i + 1][k];
                H[i][k]     = t1;
              }
            double d = std::hypot(H[k][k], H[k + 1][k]);
            cs[k]    = H[k][k] / d;
            sn[k]    = H[k + 1][k] / d;
            H[k][k]  = d;
            H[k + 1][k] = 0;
            g[k + 1] = -sn[k] * g[k];
            g[k]     = cs[k] * g[k];
            if (std::fabs(g[k + 1]) / bn <= tol * 0.5)
              {
                ++k;
                break;
              }
          }
        std::vector<double> y(k);
        for (int i = k - 1; i >= 0; --i)
          {
            double s = g[i];
            for (int j = i + 1; j < k; ++j)
              s -= H[i][j] * y[j];
            y[i] = s / H[i][i];
          }
        std::vector<double> u(n, 0.0);
        for (int i = 0; i < k; ++i)
          for (size_t t = 0; t < n; ++t)
            u[t] += y[i] * V[i][t];
        if (h->prec)
          {
            apply_preconditioner(h, u.data(), z.data());
            u.swap(z);
          }
        for (size_t t = 0; t < n; ++t)
          x[t] += u[t];
      }
    constrained_matvec(h, dense, alpha.data(), x.data(), w.data());
    for (size_t i = 0; i < n; ++i)
      r[i] = b[i] - w[i];
    rel = norm2(r) / bn;
    if (final_res)
      *final_res = rel;
    for (size_t i = 0; i < n; ++i)
      {
        if (h->dir[i] == 0)
          phi[i] = x[i];
        else
          dphi[i] = x[i];
      }
    return its;
  }

  int orc_num_blocks(orc_handle *h) { return int(h->blocks.size()); }
  int orc_num_levels(orc_handle *h) { return h->L; }
  void orc_level_range(orc_handle *h, int *s, int *e)
  {
    for (int l = 0; l <= h->L; ++l)
      {
        s[l] = h->startLevel[l];
        e[l] = h->endLevel[l];
      }
  }
  void orc_block_info(orc_handle *h, int *level, int *parent, int *nchild, double *pmin,
                      double *delta, int *n_nodes, int *n_quads)
  {
    for (size_t b = 0; b < h->blocks.size(); ++b)
      {
        const Block &B = h->blocks[b];
        level[b]       = B.level;
        parent[b]      = B.parent;
        nchild[b]      = B.nchild;
        for (int k = 0; k < 3; ++k)
          pmin[3 * b + k] = B.pmin[k];
        delta[b]   = B.delta;
        n_nodes[b] = int(B.nodes.size());
        int nq     = 0;
        for (auto &kv : B.quads)
          nq += int(kv.second.size());
        n_quads[b] = nq;
      }
  }
  int orc_childless(orc_handle *h, int *out)
  {
    for (size_t k = 0; k < h->childless.size(); ++k)
      out[k] = h->childless[k];
    return int(h->childless.size());
  }
  int orc_list_sublevels(orc_handle *h, int b) { return int(h->blocks[b].nn.size()); }
  int orc_list(orc_handle *h, int kind, int b, int sub, int *out, int cap)
  {
    const Block               &B = h->blocks[b];
    const std::vector<std::set<int>> &v = kind == 0 ? B.nn : (kind == 1 ? B.il : B.nil);
    if (sub >= int(v.size()))
      return 0;
    int k = 0;
    for (int x : v[sub])
      {
        if (k < cap)
          out[k] = x;
        ++k;
      }
    return k;
  }
  int orc_block_nodes(orc_handle *h, int b, int *out, int cap)
  {
    const Block &B = h->blocks[b];
    for (size_t k = 0; k < B.nodes.size() && int(k) < cap; ++k)
      out[k] = B.nodes[k];
    return int(B.nodes.size());
  }
  long orc_near_nnz(orc_handle *h)
  {
    long s = 0;
    for (auto &r : h->near)
      s += long(r.cols.size());
    return s;
  }
  void orc_near_export(orc_handle *h, int *rows, int *cols, double *N, double *D)
  {
    long k = 0;
    for (int i = 0; i < h->n_nodes; ++i)
      for (size_t t = 0; t < h->near[i].cols.size(); ++t, ++k)
        {
          rows[k] = i;
          cols[k] = h->near[i].cols[t];
          N[k]    = h->near[i].N[t];
          D[k]    = h->near[i].D[t];
        }
  }
  void orc_block_expansions(orc_handle *h, int kind, double *out)
  {
    const std::vector<Expansion> &E = kind == 0 ? h->M1 : kind == 1 ? h->M2 : kind == 2 ? h->L1 : h->L2;
    int                           nc = ncoef(h->p);
    for (size_t b = 0; b < E.size(); ++b)
      for (int i = 0; i < nc; ++i)
        {
          out[(b * nc + i) * 2]     = E[b].a.empty() ? 0.0 : E[b].a[i].real();
          out[(b * nc + i) * 2 + 1] = E[b].a.empty() ? 0.0 : E[b].a[i].imag();
        }
  }
  int orc_num_quad_points(orc_handle *h) { return int(h->qpts.size()); }
  void orc_quad_data(orc_handle *h, double *pts, double *nrm, double *jxw)
  {
    for (size_t k = 0; k < h->qpts.size(); ++k)
      {
        pts[3 * k]     = h->qpts[k].x;
        pts[3 * k + 1] = h->qpts[k].y;
        pts[3 * k + 2] = h->qpts[k].z;
        nrm[3 * k]     = h->qnrm[k].x;
        nrm[3 * k + 1] = h->qnrm[k].y;
        nrm[3 * k + 2] = h->qnrm[k].z;
        jxw[k]         = h->qjxw[k];
      }
  }

  double orc_legendre(int n, int m, double x)
  {
    Legendre L;
    L.eval(n, x, false);
    return L.P[tri(n, m)];
  }
  double orc_legendre_deriv(int n, int m, double x)
  {
    Legendre L;
    L.eval(n, x, true);
    return L.dS[tri(n, m)] / std::sqrt(1 - x * x);
  }

  static P3 p3(const double *x) { return P3{x[0], x[1], x[2]}; }
  static void load(Expansion &e, const double *c)
  {
    for (size_t i = 0; i < e.a.size(); ++i)
      e.a[i] = cplx(c[2 * i], c[2 * i + 1]);
    e.is_zero = false;
  }
  static void store(const Expansion &e, double *c)
  {
    for (size_t i = 0; i < e.a.size(); ++i)
      {
        c[2 * i]     = e.a[i].real();
        c[2 * i + 1] = e.a[i].imag();
      }
  }
  void orc_p2m(int p, const double *c, int npts, const double *pts, const double *q, double *out)
  {
    Expansion e(p, p3(c));
    for (int i = 0; i < npts; ++i)
      p2m_point(e, q[i], p3(pts + 3 * i));
    store(e, out);
  }
  void orc_p2m_dipole(int p, const double *c, int npts, const double *pts, const double *nrm,
                      const double *q, double *out)
  {
    Expansion e(p, p3(c));
    for (int i = 0; i < npts; ++i)
      p2m_dipole(e, q[i], p3(pts + 3 * i), p3(nrm + 3 * i));
    store(e, out);
  }
  void orc_m2m(int p, const double *cc, const double *coef, const double *cp, double *out)
  {
    Expansion ch(p, p3(cc)), par(p, p3(cp));
    load(ch, coef);
    m2m(par, ch);
    store(par, out);
  }
  void orc_m2l(int p, const double *cs, const double *coef, const double *ct, double *out)
  {
    Expansion m(p, p3(cs)), l(p, p3(ct));
    load(m, coef);
    m2l(l, m);
    store(l, out);
  }
  void orc_l2l(int p, const double *cp, const double *coef, const double *cc, double *out)
  {
    Expansion par(p, p3(cp)), ch(p, p3(cc));
    load(par, coef);
    l2l(ch, par);
    store(ch, out);
  }
  double orc_m2p(int p, const double *c, const double *coef, const double *x)
  {
    Expansion m(p, p3(c));
    load(m, coef);
    return m2p(m, p3(x));
  }
  double orc_l2p(int p, const double *c, const double *coef, const double *x)
  {
    Expansion l(p, p3(c));
    load(l, coef);
    return l2p(l, p3(x));
  }
  int orc_gauss_rule(int n, double *pts, double *w)
  {
    std::vector<double> g, gw, P, W;
    gauss01(n, g, gw);
    rule2d(g, gw, g, gw, P, W);
    std::memcpy(pts, P.data(), P.size() * sizeof(double));
    std::memcpy(w, W.data(), W.size() * sizeof(double));
    return int(W.size());
  }
  int orc_telles_rule(int n, int v, double *pts, double *w)
  {
    std::vector<double> tx, twx, ty, twy, P, W;
    telles01(n, v & 1, tx, twx);
    telles01(n, (v >> 1) & 1, ty, twy);
    rule2d(tx, twx, ty, twy, P, W);
    std::memcpy(pts, P.data(), P.size() * sizeof(double));
    std::memcpy(w, W.data(), W.size() * sizeof(double));
    return int(W.size());
  }
}
