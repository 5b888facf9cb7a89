"""C ABI on the CPU (no GPU needed): the library loads, exports every function
include/pibem_gpu.h declares, and its host-only entry points (defaults, the
.prm reader, argument validation) behave like the reference's parameter
handling (source/bem_fma.cc:65-103, source/bem_problem.cc:247-312)."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "pibem_gpu.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(pibem_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pibem_mod):
    L = pibem_mod.load()
    declared = _declared()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(pibem_mod.EXPORTS)


def test_defaults_are_the_reference_defaults(pibem_mod):
    p = pibem_mod.default_params()
    assert p.fma_truncation_order == 6
    assert p.num_octree_levels == 10
    assert p.max_nodes_per_childless_block == 20
    assert p.quadrature_order == 4
    assert p.singular_quadrature_order == 5
    assert p.gmres_restart == 100
    assert p.is_external_flow == 0
    assert p.double_body == 0
    assert p.symmetry_plane_z_level == 0.0
    assert p.continuous_gradient == 1


PRM = """
# reference layout
subsection BEMFMA<3>
  subsection FMA Params
    set FMA Truncation Order = 8
  end
  subsection Octree Params
    set Maximum Number of Collocation Points per Childless Block = 40
    set Number of Octree Levels                                  = 9
  end
end
subsection BEMProblem<3>
  set Is external flow = true
  set Solution method  = FMA
  set Symmetry plane z level = -0.25
  set Continuos gradient across edges = false
  subsection Quadrature rules
    set Quadrature order          = 3
    set Singular quadrature order = 7
  end
  subsection Solver
    set Max steps     = 321
    set Tolerance     = 1.e-9
  end
  subsection GB300 Params
    set Precision mode = Mixed
    set GMRES restart  = 60
    set HBM budget GB  = 150
    set M2L engine     = CUDA cores
    set Double body    = true
  end
end
subsection Other
  subsection Solver
    set Tolerance = 5
  end
end
"""


def test_prm_reader(pibem_mod):
    p = pibem_mod.params_from_prm(PRM)
    assert p.fma_truncation_order == 8
    assert p.max_nodes_per_childless_block == 40
    assert p.num_octree_levels == 9
    assert p.is_external_flow == 1
    assert p.quadrature_order == 3
    assert p.singular_quadrature_order == 7
    assert p.solver_max_steps == 321
    assert p.solver_tolerance == pytest.approx(1e-9)
    assert p.precision_mode == pibem_mod.PRECISION_MIXED
    assert p.gmres_restart == 60
    assert p.hbm_budget_gb == pytest.approx(150)
    assert p.m2l_engine == pibem_mod.M2L_CUDA_CORE
    assert pibem_mod.default_params().m2l_engine == pibem_mod.M2L_TENSOR_CORE
    assert p.symmetry_plane_z_level == pytest.approx(-0.25)
    assert p.double_body == 1
    assert p.continuous_gradient == 0


def test_create_rejects_bad_parameters(pibem_mod):
    L = pibem_mod.load()
    for field, bad in (("fma_truncation_order", 11), ("fma_truncation_order", 0),
                       ("num_octree_levels", 0), ("quadrature_order", 9),
                       ("singular_quadrature_order", 13), ("solver_tolerance", 0.0),
                       ("m2l_engine", 2)):
        p = pibem_mod.default_params()
        setattr(p, field, bad)
        h = C.c_void_p()
        assert L.pibem_create(C.byref(p), C.byref(h)) == pibem_mod.EINVAL
        assert not h.value


def test_null_handle_is_einval(pibem_mod):
    L = pibem_mod.load()
    assert L.pibem_set_bc(None, None) == pibem_mod.EINVAL
    assert L.pibem_destroy(None) == pibem_mod.EINVAL
    assert L.pibem_last_error(None) == b"null handle"
