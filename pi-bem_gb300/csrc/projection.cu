// L2 projections onto the continuous Q1 space of the mesh -- the steps pi-BEM
// runs on either side of the solve:
//   BEMProblem::compute_normals            (source/bem_problem.cc:1998-2070)
//   BEMProblem::compute_surface_gradients  (source/bem_problem.cc:1879-1996)
//   BEMProblem::compute_gradients          (source/bem_problem.cc:1747-1877)
// Each solves M u_c = b_c for the three components c: M_ij = sum over cells and
// Gauss points of phi_i phi_j JxW (the consistent Q1 mass matrix, the same for
// every component), b_c,i = sum phi_i g_c JxW with the projected field g =
//   the cell normal n                          (normals),
//   grad_G u = sum_b u_b grad_G phi_b          (surface gradients of u),
//   grad_G phi + n dphi/dn                     (gradients; dphi/dn interpolated),
// where grad_G phi_b = J (J^T J)^-1 grad_ref phi_b is the tangential gradient
// of the shape function through the bilinear map (J = [x_xi, x_eta], 3 x 2), as
// deal.II's FEValues gives it for a codimension-one mesh.
//
// The reference assembles M into a Trilinos matrix and solves with GMRES + AMG to
// the solver tolerance; here M is applied matrix-free from per-cell 4 x 4 blocks
// (each node gathers over its cells in a fixed order: deterministic) and the
// 3 R systems are solved together with Jacobi-preconditioned CG (M is SPD and
// well conditioned) to a relative residual of 1e-13.
#include <cmath>
#include <vector>

#include "kernels.h"
#include "krylov.h"

namespace pibem
{
  namespace
  {
    enum : int
    {
      PROJ_NORMALS = 0,
      PROJ_SURFACE_GRADIENT = 1,
      PROJ_GRADIENT = 2
    };

    // per cell: the 4 x 4 mass block and, for R columns, the 4 x 3 load vector
    // rhs[((c R + r) 4 + a) 3 + k]
    __global__ void proj_cell_kernel(int mode, int64_t n_cells, int nq, int R, int64_t N,
                                     const int32_t *__restrict__ cells,
                                     const double *__restrict__ xyz,
                                     const double *__restrict__ gpts,
                                     const double *__restrict__ qshape,
                                     const double *__restrict__ qjxw,
                                     const double *__restrict__ qnrm,
                                     const double *__restrict__ u, const double *__restrict__ dudn,
                                     double *__restrict__ cellM, double *__restrict__ rhs)
    {
      const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (c >= n_cells)
        return;
      double v[12];
      int    nd[4];
      for (int j = 0; j < 4; ++j)
        {
          nd[j] = cells[4 * c + j];
          for (int k = 0; k < 3; ++k)
            v[3 * j + k] = xyz[3 * int64_t(nd[j]) + k];
        }
      double M[16] = {};
      for (int q = 0; q < nq; ++q)
        {
          const int64_t t = c * nq + q;
          const double  w = qjxw[t];
          for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
              M[4 * a + b] += qshape[4 * t + a] * qshape[4 * t + b] * w;
        }
      for (int i = 0; i < 16; ++i)
        cellM[16 * c + i] = M[i];
      for (int r = 0; r < R; ++r)
        {
          double b[12] = {};
          for (int q = 0; q < nq; ++q)
            {
              const int64_t t = c * nq + q;
              const double  w = qjxw[t];
              double        g[3];
              if (mode == PROJ_NORMALS)
                for (int k = 0; k < 3; ++k)
                  g[k] = qnrm[3 * t + k];
              else
                {
                  const double xi = gpts[2 * q], eta = gpts[2 * q + 1];
                  double       tx[3], ty[3];
                  for (int k = 0; k < 3; ++k)
                    {
                      tx[k] = (1 - eta) * (v[3 + k] - v[k]) + eta * (v[9 + k] - v[6 + k]);
                      ty[k] = (1 - xi) * (v[6 + k] - v[k]) + xi * (v[9 + k] - v[3 + k]);
                    }
                  const double g11 = tx[0] * tx[0] + tx[1] * tx[1] + tx[2] * tx[2];
                  const double g12 = tx[0] * ty[0] + tx[1] * ty[1] + tx[2] * ty[2];
                  const double g22 = ty[0] * ty[0] + ty[1] * ty[1] + ty[2] * ty[2];
                  const double det = g11 * g22 - g12 * g12;
                  // reference gradients of the lexicographic Q1 shape functions
                  const double dxi[4]  = {-(1 - eta), 1 - eta, -eta, eta};
                  const double deta[4] = {-(1 - xi), -xi, 1 - xi, xi};
                  double       sx = 0, se = 0; // grad_ref of the interpolated u
                  for (int a = 0; a < 4; ++a)
                    {
                      const double ua = u[int64_t(r) * N + nd[a]];
                      sx += ua * dxi[a];
                      se += ua * deta[a];
                    }
                  const double cx = (g22 * sx - g12 * se) / det, ce = (-g12 * sx + g11 * se) / det;
                  for (int k = 0; k < 3; ++k)
                    g[k] = tx[k] * cx + ty[k] * ce;
                  if (mode == PROJ_GRADIENT)
                    {
                      double dn = 0;
                      for (int a = 0; a < 4; ++a)
                        dn += qshape[4 * t + a] * dudn[int64_t(r) * N + nd[a]];
                      for (int k = 0; k < 3; ++k)
                        g[k] += qnrm[3 * t + k] * dn;
                    }
                }
              for (int a = 0; a < 4; ++a)
                for (int k = 0; k < 3; ++k)
                  b[3 * a + k] += qshape[4 * t + a] * g[k] * w;
            }
          for (int i = 0; i < 12; ++i)
            rhs[(c * R + r) * 12 + i] = b[i];
        }
    }

    // For node i, visit its (cell, local vertex) incidences in a fixed order: the
    // node -> cells list is ordered by cell, a cell listed twice for a node that
    // is two vertices of a collapsed cell.
    template <typename F>
    __device__ inline void for_each_incidence(int64_t i, const int32_t *elem_off,
                                              const int32_t *elem_ids, const int32_t *cells, F f)
    {
      int prev = -1, used = -1;
      for (int e = elem_off[i]; e < elem_off[i + 1]; ++e)
        {
          const int c = elem_ids[e];
          int       from = c == prev ? used + 1 : 0, a = -1;
          for (int j = from; j < 4 && a < 0; ++j)
            if (cells[4 * int64_t(c) + j] == int(i))
              a = j;
          prev = c;
          used = a;
          if (a >= 0)
            f(c, a);
        }
    }

    // b_k[col][i] (component-major: col = 3 r + k) from the cell load vectors,
    // and the Jacobi diagonal of M
    __global__ void proj_assemble_kernel(int64_t N, int R, const int32_t *__restrict__ elem_off,
                                         const int32_t *__restrict__ elem_ids,
                                         const int32_t *__restrict__ cells,
                                         const double *__restrict__ cellM,
                                         const double *__restrict__ rhs, double *__restrict__ b,
                                         double *__restrict__ diag)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= N)
        return;
      double d = 0;
      for_each_incidence(i, elem_off, elem_ids, cells, [&](int c, int a) { d += cellM[16 * int64_t(c) + 5 * a]; });
      diag[i] = d;
      for (int r = 0; r < R; ++r)
        for (int k = 0; k < 3; ++k)
          {
            double s = 0;
            for_each_incidence(i, elem_off, elem_ids, cells, [&](int c, int a) {
              s += rhs[(int64_t(c) * R + r) * 12 + 3 * a + k];
            });
            b[(int64_t(3 * r + k)) * N + i] = s;
          }
    }

    // y[col] = M x[col] for ncol columns, matrix-free
    __global__ void proj_mass_kernel(int64_t N, int ncol, const int32_t *__restrict__ elem_off,
                                     const int32_t *__restrict__ elem_ids,
                                     const int32_t *__restrict__ cells,
                                     const double *__restrict__ cellM,
                                     const double *__restrict__ x, double *__restrict__ y)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= N)
        return;
      for (int col = 0; col < ncol; ++col)
        {
          const double *xc = x + int64_t(col) * N;
          double        s  = 0;
          for_each_incidence(i, elem_off, elem_ids, cells, [&](int c, int a) {
            const double *Mr = cellM + 16 * int64_t(c) + 4 * a;
            for (int bb = 0; bb < 4; ++bb)
              s += Mr[bb] * xc[cells[4 * int64_t(c) + bb]];
          });
          y[int64_t(col) * N + i] = s;
        }
    }

    // per column: z = r / diag ; or x += alpha p ; r -= alpha q ; p = z + beta p
    __global__ void proj_precond_kernel(int64_t N, int ncol, const double *__restrict__ diag,
                                        const double *__restrict__ r, double *__restrict__ z)
    {
      const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= N * ncol)
        return;
      z[t] = r[t] / diag[t % N];
    }

    __global__ void proj_update_kernel(int64_t N, int ncol, const double *__restrict__ alpha,
                                       const double *__restrict__ p, const double *__restrict__ q,
                                       double *__restrict__ x, double *__restrict__ r)
    {
      const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= N * ncol)
        return;
      const double a = alpha[t / N];
      x[t] += a * p[t];
      r[t] -= a * q[t];
    }

    __global__ void proj_direction_kernel(int64_t N, int ncol, const double *__restrict__ beta,
                                          const double *__restrict__ z, double *__restrict__ p)
    {
      const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= N * ncol)
        return;
      p[t] = z[t] + beta[t / N] * p[t];
    }

    // out[(r N + i) 3 + k] = x[(3 r + k) N + i]
    __global__ void proj_interleave_kernel(int64_t N, int R, const double *__restrict__ x,
                                           double *__restrict__ out)
    {
      const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= N * R * 3)
        return;
      const int64_t r = t / (3 * N), rem = t - r * 3 * N, i = rem / 3;
      const int     k = int(rem - i * 3);
      out[t]          = x[(3 * r + k) * N + i];
    }

    inline unsigned grid_for(int64_t n) { return unsigned((n + 255) / 256); }
  } // namespace

  void l2_projection(const ProjectionArgs &a, cudaStream_t s)
  {
    const int64_t N = a.n_nodes, C = a.n_cells;
    const int     R = a.R, ncol = 3 * R;
    const int64_t n = N * ncol;
    double *cellM = a.work, *rhs = cellM + 16 * C, *b = rhs + 12 * C * R, *diag = b + n,
           *x = diag + N, *r = x + n, *z = r + n, *p = z + n, *q = p + n, *part = q + n,
           *dots = part + int64_t(ncol) * 64;
    proj_cell_kernel<<<grid_for(C), 256, 0, s>>>(a.mode, C, a.nq, R, N, a.cells, a.xyz, a.gpts,
                                                  a.qshape, a.qjxw, a.qnrm, a.u, a.dudn, cellM, rhs);
    proj_assemble_kernel<<<grid_for(N), 256, 0, s>>>(N, R, a.elem_off, a.elem_ids, a.cells, cellM,
                                                      rhs, b, diag);
    PIBEM_CUDA(cudaGetLastError());
    note_launch(2);
    // Jacobi-preconditioned CG, all 3R columns together, from x = 0
    std::vector<double> bn(ncol), rz(ncol), pq(ncol), rn(ncol), al(ncol), be(ncol);
    PIBEM_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    PIBEM_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    launch_dots(N, ncol, 1, N, N, b, b, part, 64, dots, s);
    PIBEM_CUDA(cudaMemcpyAsync(bn.data(), dots, sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
    proj_precond_kernel<<<grid_for(n), 256, 0, s>>>(N, ncol, diag, r, z);
    PIBEM_CUDA(cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    launch_dots(N, ncol, 1, N, N, r, z, part, 64, dots, s);
    PIBEM_CUDA(cudaMemcpyAsync(rz.data(), dots, sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
    PIBEM_CUDA(cudaStreamSynchronize(s));
    note_launch(1);
    // A column that has converged takes no further steps (alpha = 0 leaves its
    // x and r as they are), so its result does not depend on the other columns.
    int               it = 0;
    std::vector<char> active(ncol, 1);
    for (; it < a.max_iterations; ++it)
      {
        bool done = true;
        for (int k = 0; k < ncol; ++k)
          {
            active[k] = !(rz[k] == 0 || (it > 0 && std::sqrt(rn[k]) <= a.tolerance * std::sqrt(bn[k])));
            done      = done && !active[k];
          }
        if (done)
          break;
        proj_mass_kernel<<<grid_for(N), 256, 0, s>>>(N, ncol, a.elem_off, a.elem_ids, a.cells,
                                                      cellM, p, q);
        note_launch();
        launch_dots(N, ncol, 1, N, N, p, q, part, 64, dots, s);
        PIBEM_CUDA(cudaMemcpyAsync(pq.data(), dots, sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
        PIBEM_CUDA(cudaStreamSynchronize(s));
        for (int k = 0; k < ncol; ++k)
          al[k] = active[k] && pq[k] != 0 ? rz[k] / pq[k] : 0.0;
        PIBEM_CUDA(cudaMemcpyAsync(dots, al.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, s));
        proj_update_kernel<<<grid_for(n), 256, 0, s>>>(N, ncol, dots, p, q, x, r);
        proj_precond_kernel<<<grid_for(n), 256, 0, s>>>(N, ncol, diag, r, z);
        note_launch(2);
        std::vector<double> rz_new(ncol);
        launch_dots(N, ncol, 1, N, N, r, z, part, 64, dots, s);
        PIBEM_CUDA(cudaMemcpyAsync(rz_new.data(), dots, sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
        launch_dots(N, ncol, 1, N, N, r, r, part, 64, dots + ncol, s);
        PIBEM_CUDA(cudaMemcpyAsync(rn.data(), dots + ncol, sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
        PIBEM_CUDA(cudaStreamSynchronize(s));
        for (int k = 0; k < ncol; ++k)
          {
            be[k] = rz[k] != 0 ? rz_new[k] / rz[k] : 0.0;
            rz[k] = rz_new[k];
          }
        PIBEM_CUDA(cudaMemcpyAsync(dots, be.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, s));
        proj_direction_kernel<<<grid_for(n), 256, 0, s>>>(N, ncol, dots, z, p);
        note_launch();
      }
    proj_interleave_kernel<<<grid_for(n), 256, 0, s>>>(N, R, x, a.out);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
    PIBEM_CUDA(cudaStreamSynchronize(s));
    if (a.iterations)
      *a.iterations = it;
  }

  size_t l2_projection_work(int64_t n_nodes, int64_t n_cells, int R)
  {
    const int64_t n = n_nodes * 3 * R;
    return size_t(16 * n_cells + 12 * n_cells * R + 6 * n + n_nodes + 3 * R * 64 + 6 * R);
  }
} // namespace pibem
