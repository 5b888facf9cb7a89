// Drives the C++ BEMFMA adapter (include/pibem_bemfma.hpp) the way pi-BEM's
// BEMProblem would: init_fma, octree / near field / multipole integrals, an
// FMM matvec, alpha, and a solve, on a cube-sphere read from a text file
// (n, xyz..., c, cells..., dirichlet flags..., tmp_rhs...).  Prints the solve
// statistics and the first unknowns.  A test program only.
#include <cstdio>
#include <fstream>
#include <iostream>

#include "pibem_bemfma.hpp"

int main(int argc, char **argv)
{
  if (argc < 2)
    return 2;
  std::ifstream in(argv[1]);
  long          n = 0, c = 0;
  in >> n;
  std::vector<double> xyz(3 * n);
  for (auto &v : xyz)
    in >> v;
  in >> c;
  std::vector<int32_t> cells(4 * c);
  for (auto &v : cells)
    in >> v;
  std::vector<uint8_t> dir(n);
  for (auto &v : dir)
    {
      int t;
      in >> t;
      v = uint8_t(t);
    }
  std::vector<double> tmp(n);
  for (auto &v : tmp)
    in >> v;
  try
    {
      pibem_params  p = pibem::BEMFMA::parse_parameters(
        "subsection BEMFMA<3>\n subsection FMA Params\n  set FMA Truncation Order = 4\n end\n"
        " subsection Octree Params\n  set Maximum Number of Collocation Points per Childless Block = 30\n end\nend\n");
      pibem::BEMFMA fma(&p);
      fma.init_fma(xyz, cells, std::vector<std::vector<int32_t>>(n), dir);
      fma.generate_octree_blocking();
      fma.direct_integrals();
      fma.multipole_integrals();
      std::vector<double> ones(n, 1.0), zeros(n, 0.0), oN, oD;
      fma.multipole_matr_vect_products(ones, zeros, oN, oD);
      std::vector<double> alpha = fma.compute_alpha();
      std::vector<double> phi(n), dphi(n);
      for (long i = 0; i < n; ++i)
        (dir[i] ? phi[i] : dphi[i]) = tmp[i];
      pibem_solve_stats st = fma.solve_system(phi, dphi, tmp);
      std::printf("N1[0] %.12e alpha[0] %.12e iterations %d residual %.3e\n", oN[0], alpha[0],
                  st.iterations, st.relative_residual);
      for (long i = 0; i < n; ++i)
        std::printf("%.15e %.15e\n", phi[i], dphi[i]);
    }
  catch (const pibem::Error &e)
    {
      std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
      return 1;
    }
  return 0;
}
