"""Double-node constraint lines on the GPU against the oracle (compute_constraints,
source/bem_problem.cc:1377-1579; ConstrainedOperator, include/constrained_matrix.h).

Mesh: the sharp cube (double nodes on every edge, triple nodes at the corners),
+x and +z faces Dirichlet.  Tolerances:
  * the unconstrained operator (pibem_system_matvec, BEMProblem::vmult) still
    matches the oracle's to 1e-10;
  * FP64 solves of the constrained system: within 1e-6 of the oracle's
    constrained FMM solve (same octree, lists and lines; both to 1e-10 true
    residual, the inhomogeneities of Dirichlet-Dirichlet pairs from the GPU's
    L2 projections vs the oracle's sparse direct ones);
  * mixed path within 1e-6 of the FP64 path; the solution satisfies every line
    to 1e-8 of max |x|;
  * a column's solution is the same alone and in a batch of two (bitwise)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube(synthetic):
    return synthetic.sharp_cube_case(8)


def _oracle_lines(mesh, mask, tmp, off, ids):
    import constraints
    import projections

    sets = constraints.double_sets(mesh.n_nodes, off, ids)
    nrm = projections.project(mesh.xyz, mesh.cells, "normals")
    sg = projections.project(mesh.xyz, mesh.cells, "surface_gradients", u=tmp)
    return constraints.constraint_lines(sets, mask, tmp, nrm, sg)


def _gpu(pibem_mod, cube, prec, tol=1e-10):
    mesh, mask, tmp, ph, dn, off, ids = cube
    g = pibem_mod.BEMSolver(precision_mode=prec, is_external_flow=1, fma_truncation_order=8,
                            max_nodes_per_childless_block=20, solver_tolerance=tol)
    g.set_mesh(mesh.xyz, mesh.cells, off, ids)
    g.set_bc(mask)
    return g


def test_vmult_stays_unconstrained(pibem_mod, oracle_mod, cube):
    mesh, mask, tmp, ph, dn, off, ids = cube
    g = _gpu(pibem_mod, cube, pibem_mod.PRECISION_FP64)
    o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells, off, ids)
    o.set_bc(mask)
    x = np.random.Generator(np.random.PCG64(2)).normal(size=mesh.n_nodes)
    assert rel(g.system_matvec(x), o.system_matvec(o.alpha(), x)) < 1e-10
    assert rel(g.rhs(tmp), o.rhs(o.alpha(), tmp)) < 1e-10
    g.close()


def test_constrained_solves_match_oracle(pibem_mod, oracle_mod, cube):
    mesh, mask, tmp, ph, dn, off, ids = cube
    rows, cols, gv = _oracle_lines(mesh, mask, tmp, off, ids)
    o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells, off, ids)
    o.set_bc(mask)
    o.set_constraints(rows, cols, gv)
    ophi, odphi, _, r = o.solve(tmp, tol=1e-10, max_steps=3000)
    assert r < 1e-10
    osol = np.where(mask == 1, odphi, ophi)
    sols = {}
    for prec in (pibem_mod.PRECISION_FP64, pibem_mod.PRECISION_MIXED):
        g = _gpu(pibem_mod, cube, prec)
        phi, dphi, st = g.solve(tmp)
        assert st["relative_residual"] <= 1e-10, st
        sols[prec] = np.where(mask == 1, dphi, phi)
        # alone == in a batch of two
        T = np.stack([tmp, 0.5 * tmp]).reshape(-1)
        phi2, dphi2, _ = g.solve(T)
        np.testing.assert_array_equal(phi2.reshape(2, -1)[0], phi)
        np.testing.assert_array_equal(dphi2.reshape(2, -1)[0], dphi)
        g.close()
    s64 = sols[pibem_mod.PRECISION_FP64]
    assert rel(s64, osol) < 1e-6
    assert rel(sols[pibem_mod.PRECISION_MIXED], s64) < 1e-6
    ent = cols >= 0
    scale = np.abs(s64).max()
    assert np.abs(s64[rows[ent]] - s64[cols[ent]]).max() < 1e-8 * scale
    assert np.abs(s64[rows[~ent]] - gv[~ent]).max() < 1e-6 * scale
