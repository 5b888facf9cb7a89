// pibem_bemfma.hpp -- header-only C++ adapter with the method names and call
// order of pi-BEM's BEMFMA<3> (include/bem_fma.h:94-202) and of the FMA branch
// of BEMProblem<3> (source/bem_problem.cc:1139-1374), implemented on the C ABI
// of pibem_gpu.h.  deal.II / Trilinos types are replaced by plain contiguous
// arrays (support points, cell DoF indices, full-length vectors); the INTEGRATION
// notes show the conversion at the reference's call sites.
//
// Errors are raised as pibem::Error (the reference raises deal.II exceptions
// from AssertThrow); the C ABI itself never throws.
#ifndef PIBEM_BEMFMA_HPP
#define PIBEM_BEMFMA_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pibem_gpu.h"

namespace pibem
{
  struct Error : std::runtime_error
  {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
  };

  class BEMFMA
  {
  public:
    // declare_parameters / parse_parameters (bem_fma.cc:65-103): the defaults
    // of the reference, or the knobs read from a .prm text.
    explicit BEMFMA(const pibem_params *params = nullptr)
    {
      pibem_params p;
      pibem_params_default(&p);
      if (params)
        p = *params;
      check(pibem_create(&p, &h_), nullptr);
    }
    static pibem_params parse_parameters(const std::string &prm_text)
    {
      pibem_params p;
      pibem_params_default(&p);
      pibem_params_from_prm(&p, prm_text.c_str());
      return p;
    }
    BEMFMA(const BEMFMA &)            = delete;
    BEMFMA &operator=(const BEMFMA &) = delete;
    ~BEMFMA()
    {
      if (h_)
        pibem_destroy(h_);
    }

    // BEMFMA::init_fma (bem_fma.cc:42-62): mesh, double-node sets and the
    // Dirichlet flags.  support_points: 3 per DoF; cell_dofs: 4 per Q1 cell in
    // deal.II vertex order; double_nodes: one set per DoF (may be empty).
    void init_fma(const std::vector<double> &support_points, const std::vector<int32_t> &cell_dofs,
                  const std::vector<std::vector<int32_t>> &double_nodes,
                  const std::vector<uint8_t> &dirichlet_flags)
    {
      xyz_   = support_points;
      cells_ = cell_dofs;
      dbl_off_.assign(1, 0);
      dbl_ids_.clear();
      for (const auto &s : double_nodes)
        {
          dbl_ids_.insert(dbl_ids_.end(), s.begin(), s.end());
          dbl_off_.push_back(int32_t(dbl_ids_.size()));
        }
      dir_   = dirichlet_flags;
      built_ = false;
    }

    // generate_octree_blocking + direct_integrals + multipole_integrals
    // (bem_fma.cc:3615, 108, 1609): one call builds all three on the device.
    void generate_octree_blocking() { build(); }
    void direct_integrals() { build(); }
    void multipole_integrals() { build(); }

    // generate_multipole_expansions + multipole_matr_vect_products
    // (bem_fma.cc:1971, 2391): matrVectProdN = N phi, matrVectProdD = D dphi_dn.
    void multipole_matr_vect_products(const std::vector<double> &phi,
                                      const std::vector<double> &dphi_dn,
                                      std::vector<double> &matrVectProdN,
                                      std::vector<double> &matrVectProdD)
    {
      build();
      matrVectProdN.resize(phi.size());
      matrVectProdD.resize(phi.size());
      check(pibem_fmm_matvec(h_, 1, phi.data(), dphi_dn.data(), matrVectProdN.data(),
                             matrVectProdD.data()));
    }

    // BEMProblem::compute_alpha / vmult / compute_rhs / solve_system.
    std::vector<double> compute_alpha()
    {
      build();
      std::vector<double> a(n());
      check(pibem_compute_alpha(h_, a.data()));
      return a;
    }
    void vmult(std::vector<double> &dst, const std::vector<double> &src)
    {
      build();
      dst.resize(src.size());
      check(pibem_system_matvec(h_, 1, src.data(), dst.data()));
    }
    void compute_rhs(std::vector<double> &dst, const std::vector<double> &tmp_rhs)
    {
      build();
      dst.resize(tmp_rhs.size());
      check(pibem_compute_rhs(h_, 1, tmp_rhs.data(), dst.data()));
    }
    // PreconditionILU::vmult on the matrix of BEMFMA::FMA_preconditioner
    // (bem_fma.cc:3080-3411) when the parameters ask for preconditioner 2 (the
    // leaf-block Jacobi for 1, a copy for 0): dst = P^-1 src.
    void preconditioner_vmult(std::vector<double> &dst, const std::vector<double> &src)
    {
      build();
      dst.resize(src.size());
      check(pibem_apply_preconditioner(h_, 1, src.data(), dst.data()));
    }
    pibem_solve_stats solve_system(std::vector<double> &phi, std::vector<double> &dphi_dn,
                                   const std::vector<double> &tmp_rhs)
    {
      build();
      pibem_solve_stats st{};
      check(pibem_solve(h_, 1, phi.data(), dphi_dn.data(), tmp_rhs.data(), &st));
      return st;
    }

    pibem_handle *handle() const { return h_; }
    std::size_t   n() const { return xyz_.size() / 3; }

  private:
    void build()
    {
      if (built_)
        return;
      if (xyz_.empty())
        throw Error(PIBEM_EINVAL, "init_fma was not called");
      bool any = false;
      for (std::size_t i = 0; i + 1 < dbl_off_.size(); ++i)
        any = any || dbl_off_[i + 1] > dbl_off_[i];
      check(pibem_set_mesh(h_, int64_t(n()), xyz_.data(), int64_t(cells_.size() / 4),
                           cells_.data(), any ? dbl_off_.data() : nullptr,
                           any ? dbl_ids_.data() : nullptr));
      check(pibem_set_bc(h_, dir_.data()));
      built_ = true;
    }
    void check(int rc) { check(rc, h_); }
    static void check(int rc, pibem_handle *h)
    {
      if (rc != PIBEM_OK)
        throw Error(rc, h ? pibem_last_error(h) : "pibem_create failed");
    }

    pibem_handle        *h_ = nullptr;
    std::vector<double>  xyz_;
    std::vector<int32_t> cells_, dbl_off_, dbl_ids_;
    std::vector<uint8_t> dir_;
    bool                 built_ = false;
  };
} // namespace pibem

#endif
