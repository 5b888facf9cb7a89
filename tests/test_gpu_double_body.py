"""Double body on the GPU (the reference's BEMProblem::_assemble_system_double_body,
source/bem_problem.cc:958-1135, in FMM form).

The library integrates over the mesh and its reflection in z = z0 (an FMM over
the closed geometry; image nodes carry their originals' values; only the mesh's
own nodes are collocation rows).  Tolerances:
  * every interaction in the near field (one level-1 leaf per octant): the
    operator equals the oracle's dense double body (the reference's assembly
    restated) to 1e-12;
  * regular trees: within 1e-10 of the oracle FMM of the mirrored geometry
    applied to [x, x] (same octree and lists), FP64 path;
  * alpha, rhs and vmult: 1e-10 against the same oracle;
  * solves: FP64 and mixed paths to 1e-8 true residual agree to 1e-6, are within
    the p = 8 truncation error (1e-3) of the oracle's dense double-body solve,
    and reproduce the symmetric point-source field with O(h) error;
  * the L2 projections of a double-body handle only see the mesh itself:
    bitwise the one-body handle's."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(synthetic):
    return synthetic.wigley_double_body_case(40, 8)


def _gpu(pibem_mod, mesh, mask, prec=0, **kw):
    g = pibem_mod.BEMSolver(precision_mode=prec, is_external_flow=1, double_body=1,
                            symmetry_plane_z_level=0.0, **kw)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    return g


def _oracle_mirrored(oracle_mod, mesh, mask, **kw):
    x2, c2, off, ids = oracle_mod.mirror_mesh(mesh.xyz, mesh.cells, 0.0)
    o = oracle_mod.Oracle(external=True, **kw)
    o.set_mesh(x2, c2, off, ids)
    o.set_bc(np.concatenate([mask, mask]))
    return o


def test_all_near_equals_reference_dense(pibem_mod, oracle_mod, synthetic):
    mesh, mask = synthetic.wigley_double_body_case(16, 4)[:2]
    n = mesh.n_nodes
    rng = np.random.Generator(np.random.PCG64(3))
    a, b = rng.normal(size=n), rng.normal(size=n)
    g = _gpu(pibem_mod, mesh, mask, fma_truncation_order=4, max_nodes_per_childless_block=100000)
    assert g.tree_info()["n_m2l_pairs"] == 0 and g.tree_info()["n_m2p_pairs"] == 0
    gN, gD = g.fmm_matvec(a, b)
    o = oracle_mod.Oracle(p=4, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_double_body(1, 0.0)
    oN, oD = o.dense_matvec(a, b)
    assert rel(gN, oN) < 1e-12 and rel(gD, oD) < 1e-12
    g.close()


def test_fmm_matches_oracle_of_mirrored_geometry(pibem_mod, oracle_mod, case):
    mesh, mask = case[:2]
    n = mesh.n_nodes
    g = _gpu(pibem_mod, mesh, mask, fma_truncation_order=8, max_nodes_per_childless_block=20)
    o = _oracle_mirrored(oracle_mod, mesh, mask, p=8, max_nodes=20)
    info = g.tree_info()
    assert info["n_boxes"] == len(o.tree()["level"])
    rng = np.random.Generator(np.random.PCG64(4))
    for _ in range(2):
        a, b = rng.normal(size=n), rng.normal(size=n)
        gN, gD = g.fmm_matvec(a, b)
        oN, oD = o.fmm_matvec(np.concatenate([a, a]), np.concatenate([b, b]))
        assert rel(gN, oN[:n]) < 1e-10 and rel(gD, oD[:n]) < 1e-10
    # two columns at once: the same as one at a time
    A, B = rng.normal(size=(2, n)), rng.normal(size=(2, n))
    gN2, gD2 = g.fmm_matvec(A.reshape(-1), B.reshape(-1))
    for r in range(2):
        n1, d1 = g.fmm_matvec(A[r], B[r])
        assert rel(gN2.reshape(2, n)[r], n1) < 1e-14 and rel(gD2.reshape(2, n)[r], d1) < 1e-14
    g.close()


def test_alpha_rhs_vmult_match_oracle(pibem_mod, oracle_mod, case):
    mesh, mask, tmp = case[:3]
    n = mesh.n_nodes
    g = _gpu(pibem_mod, mesh, mask, fma_truncation_order=8, max_nodes_per_childless_block=20)
    o = _oracle_mirrored(oracle_mod, mesh, mask, p=8, max_nodes=20)
    oa = o.alpha()
    assert rel(g.alpha(), oa[:n]) < 1e-10
    x = np.random.Generator(np.random.PCG64(5)).normal(size=n)
    assert rel(g.system_matvec(x), o.system_matvec(oa, np.concatenate([x, x]))[:n]) < 1e-10
    assert rel(g.rhs(tmp), o.rhs(oa, np.concatenate([tmp, tmp]))[:n]) < 1e-10
    g.close()


def test_solves(pibem_mod, oracle_mod, case):
    mesh, mask, tmp, ph, dn = case
    sols = {}
    for prec in (pibem_mod.PRECISION_FP64, pibem_mod.PRECISION_MIXED):
        g = _gpu(pibem_mod, mesh, mask, prec, fma_truncation_order=8,
                 max_nodes_per_childless_block=20, solver_tolerance=1e-8)
        phi, dphi, st = g.solve(tmp)
        assert st["relative_residual"] <= 1e-8, st
        sols[prec] = np.where(mask == 1, dphi, phi)
        g.close()
    assert rel(sols[pibem_mod.PRECISION_MIXED], sols[pibem_mod.PRECISION_FP64]) < 1e-6
    o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_double_body(1, 0.0)
    o.set_bc(mask)
    ophi, odphi, _, r = o.solve(tmp, tol=1e-10, dense=True)
    osol = np.where(mask == 1, odphi, ophi)
    assert rel(sols[pibem_mod.PRECISION_FP64], osol) < 1e-3
    exact = np.where(mask == 1, dn, ph)
    neu = mask == 0
    assert rel(sols[pibem_mod.PRECISION_FP64][neu], exact[neu]) < 0.03


def test_projections_see_the_mesh_only(pibem_mod, case):
    mesh, mask = case[:2]
    g1 = _gpu(pibem_mod, mesh, mask, fma_truncation_order=4)
    g0 = pibem_mod.BEMSolver(fma_truncation_order=4, is_external_flow=1)
    g0.set_mesh(mesh.xyz, mesh.cells)
    np.testing.assert_array_equal(g1.normals(), g0.normals())
    u = np.sin(3 * mesh.xyz[:, 0])
    np.testing.assert_array_equal(g1.surface_gradients(u), g0.surface_gradients(u))
    g1.close()
    g0.close()
