"""Properties of the oracle operator and solve (CPU): the FMM operator
converges to the dense collocation operator as the truncation order grows, the
double-layer jump gives alpha ~ 1/2 (interior) and ~ -1/2 (exterior) on a
smooth closed surface, and the solve converges to the analytic dphi/dn under
mesh refinement."""
import numpy as np

from conftest import rel


def test_fmm_converges_to_dense_with_order(oracle_mod, synthetic):
    mesh = synthetic.cube_sphere(10)
    rng = np.random.Generator(np.random.PCG64(1))
    phi, dphi = rng.normal(size=mesh.n_nodes), rng.normal(size=mesh.n_nodes)
    errs = []
    for p in (2, 4, 6, 8):
        o = oracle_mod.Oracle(p=p, levels=10, max_nodes=10)
        o.set_mesh(mesh.xyz, mesh.cells)
        fN, fD = o.fmm_matvec(phi, dphi)
        dN, dD = o.dense_matvec(phi, dphi)
        errs.append((rel(fN, dN), rel(fD, dD)))
    for a, b in zip(errs, errs[1:]):
        assert b[0] < a[0] and b[1] < a[1]
    assert errs[-1][0] < 1e-3 and errs[-1][1] < 1e-5


def test_alpha_interior_and_exterior(oracle_mod, synthetic):
    mesh = synthetic.cube_sphere(10)
    for ext, target in ((False, 0.5), (True, -0.5)):
        o = oracle_mod.Oracle(p=6, levels=10, max_nodes=20, external=ext)
        o.set_mesh(mesh.xyz, mesh.cells)
        o.set_bc(np.ones(mesh.n_nodes, np.uint8))
        a = o.alpha()
        assert abs(a.mean() - target) < 0.05


def test_solution_converges_to_analytic(oracle_mod, synthetic):
    errs = []
    for n in (6, 10, 14):
        mesh, mask, tmp, exact = synthetic.sphere_dirichlet_case(n)
        o = oracle_mod.Oracle(p=8, levels=10, max_nodes=20)
        o.set_mesh(mesh.xyz, mesh.cells)
        o.set_bc(mask)
        _, dphi, its, res = o.solve(tmp, tol=1e-10)
        assert res <= 1e-10
        errs.append(rel(dphi, exact))
    assert errs[1] < errs[0] and errs[2] < errs[1]


def test_exterior_mixed_problem_solves(oracle_mod, synthetic):
    mesh, mask, tmp, ph, dn = synthetic.spheroid_mixed_case(8, seed=2)
    o = oracle_mod.Oracle(p=6, levels=10, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_bc(mask)
    phi, dphi, its, res = o.solve(tmp, tol=1e-9)
    assert res <= 1e-9
    # unknowns against the analytic fields (coarse mesh: discretisation error)
    assert rel(np.where(mask == 0, phi, 0), np.where(mask == 0, ph, 0)) < 0.1
    assert rel(np.where(mask == 1, dphi, 0), np.where(mask == 1, dn, 0)) < 0.2
