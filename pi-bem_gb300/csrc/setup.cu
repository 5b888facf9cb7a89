// Setup kernels (FP64), run once per mesh / boundary condition:
//   quadrature data of every cell (positions, normals, JxW, shape values);
//   near-field collocation integrals (BEMFMA::direct_integrals, bem_fma.cc:108-1600)
//     with regular Gauss rules on partial cells and Telles-clustered rules on
//     singular cells;
//   P2M operator tables (BEMFMA::multipole_integrals, bem_fma.cc:1609-1840);
//   L2P evaluation tables.
#include <cmath>
#include <cstdint>
#include <mutex>

#include "devmath.cuh"
#include "kernels.h"

namespace pibem
{
  namespace
  {
    constexpr double kPi = 3.14159265358979323846;

    // Singular (Telles) rules: 4 vertices x up to 12x12 points.
    __constant__ double c_tel_pts[4][2 * 144];
    __constant__ double c_tel_w[4][144];
    __constant__ int    c_tel_n;

    // Coefficients of the normalised Legendre recurrences for n, m <= 10,
    // indexed n (n + 1) / 2 + m where two-dimensional: the square roots and the
    // reciprocal the set-up tables would otherwise evaluate per point in FP64.
    constexpr int       LEG_PMAX = 10, LEG_NPM = (LEG_PMAX + 1) * (LEG_PMAX + 2) / 2;
    __constant__ double c_leg_pm[LEG_PMAX + 1];              // -sqrt((2m - 1) / (2m))
    __constant__ double c_leg_p1[LEG_PMAX + 1];              // sqrt(2m + 1)
    __constant__ double c_leg_sq[LEG_NPM], c_leg_isq[LEG_NPM]; // sqrt((n-1)^2 - m^2), 1 / sqrt(n^2 - m^2)
    __constant__ double c_leg_d1[LEG_PMAX + 1];              // sqrt(n (n + 1))
    __constant__ double c_leg_d2[LEG_NPM], c_leg_d3[LEG_NPM]; // sqrt((n-m)(n+m+1)), sqrt((n+m)(n-m+1))

    struct Geo
    {
      double x[3], n[3], J, N[4];
    };

    // Bilinear map of a Q1 cell; the position is summed in a fixed order
    // without fused multiply-adds (matches the oracle bit for bit).
    __device__ inline void cell_geo(const double *v, double xi, double eta, Geo &g)
    {
      const double a0 = __dmul_rn(__dadd_rn(1.0, -xi), __dadd_rn(1.0, -eta));
      const double a1 = __dmul_rn(xi, __dadd_rn(1.0, -eta));
      const double a2 = __dmul_rn(__dadd_rn(1.0, -xi), eta);
      const double a3 = __dmul_rn(xi, eta);
      g.N[0] = a0;
      g.N[1] = a1;
      g.N[2] = a2;
      g.N[3] = a3;
      for (int k = 0; k < 3; ++k)
        {
          double s = __dadd_rn(__dmul_rn(v[0 * 3 + k], a0), __dmul_rn(v[1 * 3 + k], a1));
          s        = __dadd_rn(s, __dmul_rn(v[2 * 3 + k], a2));
          s        = __dadd_rn(s, __dmul_rn(v[3 * 3 + k], a3));
          g.x[k]   = s;
        }
      double tx[3], ty[3];
      for (int k = 0; k < 3; ++k)
        {
          tx[k] = (1 - eta) * (v[3 + k] - v[k]) + eta * (v[9 + k] - v[6 + k]);
          ty[k] = (1 - xi) * (v[6 + k] - v[k]) + xi * (v[9 + k] - v[3 + k]);
        }
      double c[3] = {tx[1] * ty[2] - tx[2] * ty[1], tx[2] * ty[0] - tx[0] * ty[2],
                     tx[0] * ty[1] - tx[1] * ty[0]};
      g.J         = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      for (int k = 0; k < 3; ++k)
        g.n[k] = c[k] / g.J;
    }

    __global__ void quad_data_kernel(int64_t n_cells, int nq, const double *__restrict__ xyz,
                                     const int32_t *__restrict__ cells,
                                     const double *__restrict__ gpts,
                                     const double *__restrict__ gw, double *qpts, double *qnrm,
                                     double *qjxw, double *qshape)
    {
      int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= n_cells * nq)
        return;
      int64_t c = t / nq;
      int     q = int(t % nq);
      double  v[12];
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k)
          v[3 * j + k] = xyz[3 * int64_t(cells[4 * c + j]) + k];
      Geo g;
      cell_geo(v, gpts[2 * q], gpts[2 * q + 1], g);
      for (int k = 0; k < 3; ++k)
        {
          qpts[3 * t + k] = g.x[k];
          qnrm[3 * t + k] = g.n[k];
        }
      qjxw[t] = g.J * gw[q];
      for (int j = 0; j < 4; ++j)
        qshape[4 * t + j] = g.N[j];
    }

    // LaplaceKernel::kernels (include/laplace_kernel.h:55-74) contracted with
    // the normal: s = 1 / (4 pi r), dn = D.n with D = R / (-4 pi r^3), from one
    // reciprocal square root (FP64 division and square root are
    // multi-instruction sequences on the FP64 pipe, which bounds this kernel)
    __device__ inline void kernel_pair(const double *R, const double *n, double &dn, double &s)
    {
      constexpr double c4pi = 1.0 / (4 * kPi);
      const double     r2   = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
      const double     rinv = rsqrt(r2);
      s                     = rinv * c4pi;
      dn                    = -(R[0] * n[0] + R[1] * n[1] + R[2] * n[2]) * (rinv * rinv * rinv) * c4pi;
    }

    // One (leaf row, entry) integral: 4 N values and 4 D values.  PASS 0 takes
    // the items of a batch, integrates the regular ones (Gauss points) and
    // lists the singular ones (the cell holds the row's node or a double of
    // it); PASS 1 integrates the listed items (Telles rule), so that a warp's
    // threads run the same rule (a singular item costs several times a regular
    // one).  Every item's values depend on the item alone.
    template <int PASS>
    __global__ void near_entries_kernel(int64_t n_items, int n_leaves,
                                        const int64_t *__restrict__ item_ptr,
                                        const int64_t *__restrict__ row_ptr,
                                        const int64_t *__restrict__ ent_ptr,
                                        const int32_t *__restrict__ rows,
                                        const NearEntry *__restrict__ ents,
                                        const double *__restrict__ xyz,
                                        const int32_t *__restrict__ cells,
                                        const int32_t *__restrict__ dbl_off,
                                        const int32_t *__restrict__ dbl_ids, int nq,
                                        const double *__restrict__ qpts,
                                        const double *__restrict__ qnrm,
                                        const double *__restrict__ qjxw,
                                        const double *__restrict__ qshape, int64_t item_base,
                                        double *__restrict__ staging,
                                        int64_t *__restrict__ sing_list,
                                        unsigned long long *__restrict__ sing_count)
    {
      auto item = [&](int64_t it) {
        // leaf by binary search over item_ptr
        int lo = 0, hi = n_leaves - 1;
        while (lo < hi)
          {
            int mid = (lo + hi + 1) >> 1;
            if (item_ptr[mid] <= it)
              lo = mid;
            else
              hi = mid - 1;
          }
        const int     leaf = lo;
        const int64_t loc  = it - item_ptr[leaf];
        const int64_t ne   = ent_ptr[leaf + 1] - ent_ptr[leaf];
        const int64_t r    = loc / ne;
        const int64_t e    = loc % ne;
        const int     node = rows[row_ptr[leaf] + r];
        const NearEntry E  = ents[ent_ptr[leaf] + e];
        const int64_t   c  = E.cell;
        double xi[3] = {xyz[3 * int64_t(node)], xyz[3 * int64_t(node) + 1], xyz[3 * int64_t(node) + 2]};
        double Nv[4] = {0, 0, 0, 0}, Dv[4] = {0, 0, 0, 0};
        int    sv = -1;
        if (E.singular_ok)
          for (int j = 0; j < 4 && sv < 0; ++j)
            {
              int d = cells[4 * c + j];
              for (int a = dbl_off[node]; a < dbl_off[node + 1]; ++a)
                if (dbl_ids[a] == d)
                  {
                    sv = j;
                    break;
                  }
            }
        if (PASS == 0 && sv >= 0)
          {
            sing_list[atomicAdd(sing_count, 1ull)] = it;
            return;
          }
        if (sv < 0)
          {
            uint64_t mask = E.qmask;
            while (mask)
              {
                int q = __ffsll((long long)mask) - 1;
                mask &= mask - 1;
                int64_t k = c * nq + q;
                double  R[3] = {qpts[3 * k] - xi[0], qpts[3 * k + 1] - xi[1], qpts[3 * k + 2] - xi[2]};
                double  n[3] = {qnrm[3 * k], qnrm[3 * k + 1], qnrm[3 * k + 2]};
                double  dn, s;
                kernel_pair(R, n, dn, s);
                double w = qjxw[k];
                for (int j = 0; j < 4; ++j)
                  {
                    Nv[j] += dn * qshape[4 * k + j] * w;
                    Dv[j] += s * qshape[4 * k + j] * w;
                  }
              }
          }
        else
          {
            double v[12];
            for (int j = 0; j < 4; ++j)
              for (int k = 0; k < 3; ++k)
                v[3 * j + k] = xyz[3 * int64_t(cells[4 * c + j]) + k];
            const int nt = c_tel_n;
            for (int q = 0; q < nt; ++q)
              {
                Geo g;
                cell_geo(v, c_tel_pts[sv][2 * q], c_tel_pts[sv][2 * q + 1], g);
                double R[3] = {g.x[0] - xi[0], g.x[1] - xi[1], g.x[2] - xi[2]};
                double dn, s;
                kernel_pair(R, g.n, dn, s);
                double w = g.J * c_tel_w[sv][q];
                for (int j = 0; j < 4; ++j)
                  {
                    Nv[j] += dn * g.N[j] * w;
                    Dv[j] += s * g.N[j] * w;
                  }
              }
          }
        double *o = staging + (it - item_base) * 8;
        for (int j = 0; j < 4; ++j)
          {
            o[j]     = Nv[j];
            o[4 + j] = Dv[j];
          }
      };
      const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (PASS == 0)
        {
          if (item_base + g < n_items)
            item(item_base + g);
        }
      else
        {
          const int64_t cnt = int64_t(*sing_count);
          for (int64_t q = g; q < cnt; q += int64_t(gridDim.x) * blockDim.x)
            item(sing_list[q]);
        }
    }

    // Deterministic gather of the entry integrals into the dense leaf blocks.
    __global__ void near_gather_kernel(int64_t n_vals, int n_leaves,
                                       const int64_t *__restrict__ val_ptr,
                                       const int64_t *__restrict__ col_ptr,
                                       const int64_t *__restrict__ ent_ptr,
                                       const int64_t *__restrict__ item_ptr,
                                       const int32_t *__restrict__ gather_ptr,
                                       const int32_t *__restrict__ gather_ids, int64_t item_base,
                                       int64_t item_end, const double *__restrict__ staging,
                                       double *__restrict__ Nval, double *__restrict__ Dval,
                                       int64_t val_base)
    {
      int64_t vi = val_base + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (vi >= n_vals)
        return;
      int lo = 0, hi = n_leaves - 1;
      while (lo < hi)
        {
          int mid = (lo + hi + 1) >> 1;
          if (val_ptr[mid] <= vi)
            lo = mid;
          else
            hi = mid - 1;
        }
      const int     leaf = lo;
      const int64_t nc   = col_ptr[leaf + 1] - col_ptr[leaf];
      const int64_t ld   = (nc + 3) / 4 * 4; // padded row stride
      const int64_t ne   = ent_ptr[leaf + 1] - ent_ptr[leaf];
      const int64_t loc  = vi - val_ptr[leaf];
      const int64_t r    = loc / ld;
      const int64_t cc   = loc % ld;
      if (cc >= nc)
        return; // padding (stays zero)
      const int64_t gcol = col_ptr[leaf] + cc;
      const int64_t ib   = item_ptr[leaf] + r * ne;
      if (ib < item_base || ib + ne > item_end)
        return; // not in this batch
      double sn = 0, sd = 0;
      for (int g = gather_ptr[gcol]; g < gather_ptr[gcol + 1]; ++g)
        {
          int     id = gather_ids[g];
          int64_t e = id >> 2, j = id & 3;
          const double *st = staging + (ib + e - item_base) * 8;
          sn += st[j];
          sd += st[4 + j];
        }
      Nval[vi] = sn;
      Dval[vi] = sd;
    }

    // P2M tables: for P2M row (leaf, dof) the scaled expansion (K reals) of the
    // dipole layer (Ker1, MultipoleExpansion::AddNormDer multipole_expansion.cc:125-181)
    // and of the single layer (Ker2, MultipoleExpansion::Add multipole_expansion.cc:94-122)
    // of the dof's shape function over the leaf's quadrature points, strengths
    // N_j JxW / (4 pi) (bem_fma.cc:1722-1734).  One block per row: the row's
    // contributions are taken P2M_CHUNK at a time; per contribution one thread
    // computes its geometry (scaled offset, angles, normal derivatives of rho,
    // alpha, beta), rho^n, cos / sin (m beta) and the tables of P~_n^m and
    // dP~_n^m/dtheta into shared memory, then thread k adds the contributions'
    // terms of coefficient k in contribution order.
    // P~_n^m(x) of every n <= p, m <= n into P[n (n + 1) / 2 + m] and, with dS,
    // legendre_dsin(n, m) into dS[...]: the recurrences of legendre_nm and
    // legendre_dsin (devmath.cuh) at O(p^2), their square-root factors from
    // the constant tables (the same values) and the division of the
    // three-term recurrence as a product with the reciprocal (the values agree
    // with theirs to a few ulp).
    __device__ inline void legendre_table(int p, double x, double s, double *P, double *dS)
    {
      double pmm = 1.0;
      for (int m = 0; m <= p; ++m)
        {
          if (m > 0)
            pmm *= c_leg_pm[m] * s;
          P[m * (m + 1) / 2 + m] = pmm;
          if (m + 1 > p)
            continue;
          double p1 = x * c_leg_p1[m] * pmm, p0 = pmm;
          P[(m + 1) * (m + 2) / 2 + m] = p1;
          for (int n = m + 2; n <= p; ++n)
            {
              const int    nm = n * (n + 1) / 2 + m;
              const double p2 = (double(2 * n - 1) * x * p1 - c_leg_sq[nm] * p0) * c_leg_isq[nm];
              p0              = p1;
              p1              = p2;
              P[nm]           = p2;
            }
        }
      if (!dS)
        return;
      for (int n = 0; n <= p; ++n)
        for (int m = 0; m <= n; ++m)
          {
            auto   pv = [&](int mm) { return mm >= 0 && mm <= n ? P[n * (n + 1) / 2 + mm] : 0.0; };
            const int nm = n * (n + 1) / 2 + m;
            double dth;
            if (m == 0)
              dth = n > 0 ? c_leg_d1[n] * pv(1) : 0.0;
            else
              dth = 0.5 * (c_leg_d2[nm] * pv(m + 1) - c_leg_d3[nm] * pv(m - 1));
            dS[nm] = -dth;
          }
    }

    constexpr int P2M_CHUNK = 32;
    // doubles per contribution in shared memory for order p
    __host__ __device__ inline int p2m_geo_stride(int p)
    {
      const int npm = (p + 1) * (p + 2) / 2;
      return 8 + 3 * (p + 1) + 2 * npm;
    }
    __global__ void __launch_bounds__(128)
      p2m_table_kernel(int64_t n_rows, int K, int p, int n_leaves,
                       const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ leaf_box,
                       const int64_t *__restrict__ contrib_ptr,
                       const int32_t *__restrict__ contrib_q,
                       const double *__restrict__ box_center,
                       const double *__restrict__ box_delta, const double *__restrict__ qpts,
                       const double *__restrict__ qnrm, const double *__restrict__ qjxw,
                       const double *__restrict__ qshape, double *T1, double *T2)
    {
      extern __shared__ double geo[]; // [P2M_CHUNK][stride]
      const int64_t row = blockIdx.x;
      if (row >= n_rows)
        return;
      const int stride = p2m_geo_stride(p);
      const int npm    = (p + 1) * (p + 2) / 2;
      // layout of one contribution: 0 w, 1 ws, 2 rho, 3 dRhodN, 4 dBetadN,
      // 5 dAlphadN, 6 ca, 7 sa, then rn[p+1], cos(m beta)[p+1], sin(m beta)[p+1],
      // P[npm], dS[npm] (pair (n, m) at n (n+1) / 2 + m)
      int lo = 0, hi = n_leaves - 1;
      while (lo < hi)
        {
          int mid = (lo + hi + 1) >> 1;
          if (row_ptr[mid] <= row)
            lo = mid;
          else
            hi = mid - 1;
        }
      const int    box = leaf_box[lo];
      const double h   = box_delta[box];
      const double cx = box_center[3 * box], cy = box_center[3 * box + 1],
                   cz = box_center[3 * box + 2];
      const int k = threadIdx.x;
      int       n = 0, m = 0, part = 0;
      if (k < K)
        real_index(k, n, m, part);
      double        a1 = 0, a2 = 0;
      const int64_t c0 = contrib_ptr[row], c1 = contrib_ptr[row + 1];
      for (int64_t cb0 = c0; cb0 < c1; cb0 += P2M_CHUNK)
        {
          const int nc = int(c1 - cb0 < P2M_CHUNK ? c1 - cb0 : int64_t(P2M_CHUNK));
          __syncthreads(); // the previous chunk's values are used up
          if (threadIdx.x < nc)
            {
              double       *gq = geo + threadIdx.x * stride;
              const int32_t qj = contrib_q[cb0 + threadIdx.x];
              const int64_t q  = qj >> 2;
              const int     j  = qj & 3;
              const double  w  = qshape[4 * q + j] * qjxw[q] / 4 / kPi;
              const double  rx = (qpts[3 * q] - cx) / h, ry = (qpts[3 * q + 1] - cy) / h,
                           rz = (qpts[3 * q + 2] - cz) / h;
              const double rho  = sqrt(rx * rx + ry * ry + rz * rz);
              const double ca   = rz / rho;
              const double sa   = sqrt(fmax(0.0, 1.0 - ca * ca));
              const double beta = atan2(ry, rx);
              double nn_ = sqrt(qnrm[3 * q] * qnrm[3 * q] + qnrm[3 * q + 1] * qnrm[3 * q + 1] +
                                qnrm[3 * q + 2] * qnrm[3 * q + 2]);
              double nx = qnrm[3 * q] / nn_, ny = qnrm[3 * q + 1] / nn_, nz = qnrm[3 * q + 2] / nn_;
              double rxy2 = rx * rx + ry * ry;
              gq[0]       = w;
              gq[1]       = w / h;
              gq[2]       = rho;
              gq[3]       = (rx / rho) * nx + (ry / rho) * ny + (rz / rho) * nz;
              gq[4]       = (-ry / rxy2) * nx + (rx / rxy2) * ny;
              gq[5] = (ca * cos(beta) / rho) * nx + (ca * sin(beta) / rho) * ny + (-sa / rho) * nz;
              gq[6] = ca;
              gq[7] = sa;
              double rn = 1.0;
              for (int i = 0; i <= p; ++i)
                {
                  gq[8 + i] = rn;
                  rn *= rho;
                }
              for (int mm = 0; mm <= p; ++mm)
                {
                  double sb, cb;
                  sincos(mm * beta, &sb, &cb);
                  gq[8 + (p + 1) + mm]     = cb;
                  gq[8 + 2 * (p + 1) + mm] = sb;
                }
              legendre_table(p, ca, sa, gq + 8 + 3 * (p + 1), gq + 8 + 3 * (p + 1) + npm);
            }
          __syncthreads();
          if (k < K)
            for (int cq = 0; cq < nc; ++cq)
              {
                const double *gq  = geo + cq * stride;
                const int     pmi = n * (n + 1) / 2 + m;
                const double  cb = gq[8 + (p + 1) + m], sb = gq[8 + 2 * (p + 1) + m];
                const double  P  = gq[8 + 3 * (p + 1) + pmi];
                const double  rn = gq[8 + n];
                // monopole: w P rho^n e^{-i m beta}
                const double mono = gq[0] * P * rn;
                a2 += part == 0 ? mono * cb : -mono * sb;
                // dipole (scaled coordinates, strength w / h)
                const double dS   = gq[8 + 3 * (p + 1) + npm + pmi];
                const double rho  = gq[2];
                const double rnm1 = n > 0 ? rn / rho : 0.0;
                const double A    = double(n) * rnm1 * P * gq[3] - rn * dS * gq[5];
                const double B    = -double(m) * rn * P * gq[4];
                // e^{-i m beta} (A + i B)
                a1 += gq[1] * (part == 0 ? (cb * A + sb * B) : (cb * B - sb * A));
              }
        }
      if (k < K)
        {
          const int K4    = (K + 3) / 4 * 4; // padded row stride (16-byte vector loads)
          T1[row * K4 + k] = a1;
          T2[row * K4 + k] = a2;
        }
    }

    // L2P tables: W[pos][k] such that the field at node rows[pos] of its leaf is
    // sum_k W[pos][k] L^[leaf][k] (LocalExpansion::Evaluate local_expansion.cc:252-287).
    // One warp per position: lane 0 forms the geometry and the Legendre table,
    // the lanes cos / sin (m beta) and then the K coefficients.
    __global__ void __launch_bounds__(256)
      l2p_table_kernel(int64_t n_pos, int K, int p, int ldw, int n_leaves,
                       const int64_t *__restrict__ pos_ptr, const int32_t *__restrict__ leaf_box,
                       const int32_t *__restrict__ nodes, const double *__restrict__ xyz,
                       const double *__restrict__ box_center,
                       const double *__restrict__ box_delta, double *W)
    {
      extern __shared__ double lgeo[]; // per warp: [rho, ca, sa, beta, h | rn[p+1] | cos[p+1] | sin[p+1] | P[npm]]
      const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const int64_t pos  = int64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
      const int     npm  = (p + 1) * (p + 2) / 2;
      double       *g    = lgeo + warp * (5 + 3 * (p + 1) + npm);
      if (pos >= n_pos)
        return;
      int lo = 0, hi = n_leaves - 1;
      while (lo < hi)
        {
          int mid = (lo + hi + 1) >> 1;
          if (pos_ptr[mid] <= pos)
            lo = mid;
          else
            hi = mid - 1;
        }
      const int    box  = leaf_box[lo];
      const double h    = box_delta[box];
      const int    node = nodes[pos];
      if (lane == 0)
        {
          const double rx  = (xyz[3 * int64_t(node)] - box_center[3 * box]) / h;
          const double ry  = (xyz[3 * int64_t(node) + 1] - box_center[3 * box + 1]) / h;
          const double rz  = (xyz[3 * int64_t(node) + 2] - box_center[3 * box + 2]) / h;
          const double rho = sqrt(rx * rx + ry * ry + rz * rz);
          g[0]             = rho;
          if (rho > 0)
            {
              const double ca   = rz / rho;
              const double sa   = sqrt(fmax(0.0, 1.0 - ca * ca));
              const double beta = atan2(ry, rx);
              g[1]              = ca;
              g[2]              = sa;
              g[3]              = beta;
              double rn         = 1.0;
              for (int i = 0; i <= p; ++i)
                {
                  g[5 + i] = rn;
                  rn *= rho;
                }
            }
        }
      __syncwarp();
      const double rho = g[0];
      if (rho > 0)
        {
          for (int mm = lane; mm <= p; mm += 32)
            {
              double sb, cb;
              sincos(mm * g[3], &sb, &cb);
              g[5 + (p + 1) + mm]     = cb;
              g[5 + 2 * (p + 1) + mm] = sb;
            }
          if (lane == 0)
            legendre_table(p, g[1], g[2], g + 5 + 3 * (p + 1), nullptr);
        }
      __syncwarp();
      for (int k = lane; k < K; k += 32)
        {
          int n, m, part;
          real_index(k, n, m, part);
          double val = 0.0;
          if (rho > 0)
            {
              const double cb = g[5 + (p + 1) + m], sb = g[5 + 2 * (p + 1) + m];
              const double P  = g[5 + 3 * (p + 1) + n * (n + 1) / 2 + m] * g[5 + n];
              if (m == 0)
                val = P;
              else
                val = part == 0 ? 2.0 * P * cb : -2.0 * P * sb;
            }
          else if (k == 0)
            val = 1.0;
          W[pos * ldw + k] = val / h;
        }
    }
  } // namespace

  void set_telles_rules(const std::vector<double> pts[4], const std::vector<double> w[4], int n,
                        cudaStream_t s)
  {
    double hp[4][2 * 144] = {}, hw[4][144] = {};
    for (int v = 0; v < 4; ++v)
      for (int q = 0; q < n; ++q)
        {
          hp[v][2 * q]     = pts[v][2 * q];
          hp[v][2 * q + 1] = pts[v][2 * q + 1];
          hw[v][q]         = w[v][q];
        }
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_tel_pts, hp, sizeof(hp), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_tel_w, hw, sizeof(hw), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_tel_n, &n, sizeof(int), 0, cudaMemcpyHostToDevice, s));
  }

  void launch_quad_data(int64_t n_cells, int nq, const double *xyz, const int32_t *cells,
                        const double *gpts, const double *gw, double *qpts, double *qnrm,
                        double *qjxw, double *qshape, cudaStream_t s)
  {
    int64_t n = n_cells * nq;
    if (n == 0)
      return;
    quad_data_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n_cells, nq, xyz, cells, gpts, gw,
                                                               qpts, qnrm, qjxw, qshape);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_near_assembly(const NearAssemblyArgs &a, cudaStream_t s)
  {
    // batches bounded by the staging buffer (items of 8 doubles)
    const int64_t n_items = a.n_items;
    int64_t       start   = 0;
    while (start < n_items)
      {
        // extend the batch to whole (leaf,row) groups: find the leaf boundary
        int64_t end = std::min(n_items, start + a.staging_items);
        if (end < n_items)
          {
            // move end back to a row boundary of its leaf
            int lo = 0, hi = a.n_leaves - 1;
            while (lo < hi)
              {
                int mid = (lo + hi + 1) >> 1;
                if (a.h_item_ptr[mid] <= end)
                  lo = mid;
                else
                  hi = mid - 1;
              }
            int64_t ne  = a.h_ent_ptr[lo + 1] - a.h_ent_ptr[lo];
            int64_t rb  = a.h_item_ptr[lo] + ((end - a.h_item_ptr[lo]) / ne) * ne;
            if (rb <= start)
              throw Error(PIBEM_ENOMEM_HBM, "near-field staging buffer too small for one row");
            end = rb;
          }
        int64_t cnt = end - start;
        PIBEM_CUDA(cudaMemsetAsync(a.sing_count, 0, sizeof(unsigned long long), s));
        near_entries_kernel<0><<<unsigned((cnt + 127) / 128), 128, 0, s>>>(
          end, a.n_leaves, a.item_ptr, a.row_ptr, a.ent_ptr, a.rows, a.ents, a.xyz, a.cells,
          a.dbl_off, a.dbl_ids, a.nq, a.qpts, a.qnrm, a.qjxw, a.qshape, start, a.staging,
          a.sing_list, a.sing_count);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
        // the singular items of the batch (a grid-stride loop over the list)
        near_entries_kernel<1><<<unsigned(std::min<int64_t>((cnt + 127) / 128, 4096)), 128, 0, s>>>(
          end, a.n_leaves, a.item_ptr, a.row_ptr, a.ent_ptr, a.rows, a.ents, a.xyz, a.cells,
          a.dbl_off, a.dbl_ids, a.nq, a.qpts, a.qnrm, a.qjxw, a.qshape, start, a.staging,
          a.sing_list, a.sing_count);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
        // gather: all values whose row lies in [start, end)
        // value range: leaves covering the batch
        int l0 = 0, hi = a.n_leaves - 1;
        {
          int lo = 0;
          hi     = a.n_leaves - 1;
          while (lo < hi)
            {
              int mid = (lo + hi + 1) >> 1;
              if (a.h_item_ptr[mid] <= start)
                lo = mid;
              else
                hi = mid - 1;
            }
          l0 = lo;
        }
        int l1 = l0;
        while (l1 + 1 < a.n_leaves && a.h_item_ptr[l1 + 1] < end)
          ++l1;
        int64_t v0 = a.h_val_ptr[l0], v1 = a.h_val_ptr[l1 + 1];
        int64_t nv = v1 - v0;
        if (nv > 0)
          near_gather_kernel<<<unsigned((nv + 255) / 256), 256, 0, s>>>(
            v1, a.n_leaves, a.val_ptr, a.col_ptr, a.ent_ptr, a.item_ptr, a.gather_ptr,
            a.gather_ids, start, end, a.staging, a.Nval, a.Dval, v0);
        PIBEM_CUDA(cudaGetLastError());
    note_launch();
        start = end;
      }
  }

  // The Legendre coefficient tables in constant memory, once per device.
  static void set_legendre_coeffs(cudaStream_t s)
  {
    static std::mutex mu;
    static bool       done[64] = {};
    int               dev      = 0;
    PIBEM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 64 && done[dev])
      return;
    double pm[LEG_PMAX + 1] = {}, p1[LEG_PMAX + 1] = {}, d1[LEG_PMAX + 1] = {};
    double sq[LEG_NPM] = {}, isq[LEG_NPM] = {}, d2[LEG_NPM] = {}, d3[LEG_NPM] = {};
    for (int m = 0; m <= LEG_PMAX; ++m)
      {
        pm[m] = m > 0 ? -std::sqrt(double(2 * m - 1) / double(2 * m)) : 0.0;
        p1[m] = std::sqrt(double(2 * m + 1));
        d1[m] = std::sqrt(double(m) * double(m + 1));
      }
    for (int n = 0; n <= LEG_PMAX; ++n)
      for (int m = 0; m <= n; ++m)
        {
          const int nm = n * (n + 1) / 2 + m;
          if (n >= m + 2)
            {
              sq[nm]  = std::sqrt(double((n - 1) * (n - 1) - m * m));
              isq[nm] = 1.0 / std::sqrt(double(n * n - m * m));
            }
          d2[nm] = std::sqrt(double(n - m) * double(n + m + 1));
          d3[nm] = std::sqrt(double(n + m) * double(n - m + 1));
        }
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_pm, pm, sizeof(pm), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_p1, p1, sizeof(p1), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_d1, d1, sizeof(d1), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_sq, sq, sizeof(sq), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_isq, isq, sizeof(isq), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_d2, d2, sizeof(d2), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg_d3, d3, sizeof(d3), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaStreamSynchronize(s)); // the host arrays go out of scope
    if (dev < 64)
      done[dev] = true;
  }

  void launch_p2m_tables(int64_t n_rows, int K, int p, int n_leaves, const int64_t *row_ptr,
                         const int32_t *leaf_box, const int64_t *contrib_ptr,
                         const int32_t *contrib_q, const double *box_center,
                         const double *box_delta, const double *qpts, const double *qnrm,
                         const double *qjxw, const double *qshape, double *T1, double *T2,
                         cudaStream_t s)
  {
    int64_t n = n_rows * K;
    if (n == 0)
      return;
    if (K > 128 || p > LEG_PMAX)
      throw Error(PIBEM_EINVAL, "P2M tables: more than 128 coefficients");
    set_legendre_coeffs(s);
    const size_t smem = size_t(P2M_CHUNK) * p2m_geo_stride(p) * sizeof(double);
    if (smem > 48 * 1024)
      raise_smem_limit(reinterpret_cast<const void *>(p2m_table_kernel), smem);
    p2m_table_kernel<<<unsigned(n_rows), 128, smem, s>>>(
      n_rows, K, p, n_leaves, row_ptr, leaf_box, contrib_ptr, contrib_q, box_center, box_delta,
      qpts, qnrm, qjxw, qshape, T1, T2);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_l2p_tables(int64_t n_pos, int K, int ldw, int n_leaves, const int64_t *pos_ptr,
                         const int32_t *leaf_box, const int32_t *nodes, const double *xyz,
                         const double *box_center, const double *box_delta, double *W,
                         cudaStream_t s)
  {
    if (n_pos == 0)
      return;
    int p = 0;
    while ((p + 1) * (p + 1) < K)
      ++p;
    if (p > LEG_PMAX)
      throw Error(PIBEM_EINVAL, "L2P tables: order above 10");
    set_legendre_coeffs(s);
    const size_t smem = size_t(8) * (5 + 3 * (p + 1) + (p + 1) * (p + 2) / 2) * sizeof(double);
    l2p_table_kernel<<<unsigned((n_pos + 7) / 8), 256, smem, s>>>(n_pos, K, p, ldw, n_leaves,
                                                                  pos_ptr, leaf_box, nodes, xyz,
                                                                  box_center, box_delta, W);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
} // namespace pibem
