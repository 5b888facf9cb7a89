"""The FP64-accurate operator with float-float (FP32-pair) translations and the
tcgen05 BF16-digit M2L against the plain FP64 operator and the oracle's operator
(BEMProblem::vmult / compute_rhs restated on the CPU), through the C ABI:
operator applications agree with the FP64 operator to 1e-12 and with the oracle
to 1e-11 relative (2-norm) at p = 6, 8, 10, and solves in that mode meet the
FP64 residual and agree with the FP64 path's solution to 1e-9."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

CASES = [
    ("perturbed_p6", dict(n=12, p=6, leaf=16, perturbed=True)),
    ("spheroid_p8", dict(n=20, p=8, leaf=40)),
    ("spheroid_p10", dict(n=16, p=10, leaf=30)),
]


def _case(S, c):
    if c.get("perturbed"):
        mesh = S.perturbed_sphere(c["n"], seed=11)
        return S.spheroid_mixed_case(0, seed=4, mesh=mesh)[:3]
    return S.spheroid_mixed_case(c["n"], seed=2)[:3]


def _handle(pibem, c, mesh, mask, mode, tol=1e-8):
    g = pibem.BEMSolver(fma_truncation_order=c["p"], max_nodes_per_childless_block=c["leaf"],
                        is_external_flow=1, precision_mode=mode, solver_tolerance=tol)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    return g


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
def test_float_float_operator(name, c, pibem_mod, synthetic, oracle_mod):
    mesh, mask, tmp = _case(synthetic, c)
    x = np.random.Generator(np.random.PCG64(9)).normal(size=(2, mesh.n_nodes)).reshape(-1)
    g64 = _handle(pibem_mod, c, mesh, mask, pibem_mod.PRECISION_FP64, 1e-11)
    gff = _handle(pibem_mod, c, mesh, mask, pibem_mod.PRECISION_FLOAT_FLOAT, 1e-11)
    assert rel(gff.system_matvec(x), g64.system_matvec(x)) < 1e-12
    assert rel(gff.rhs(tmp), g64.rhs(tmp)) < 1e-12
    n1, d1 = gff.fmm_matvec(x, x[::-1].copy())
    n2, d2 = g64.fmm_matvec(x, x[::-1].copy())
    assert rel(n1, n2) < 1e-12 and rel(d1, d2) < 1e-12
    o = oracle_mod.Oracle(p=c["p"], levels=10, max_nodes=c["leaf"], external=True)
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_bc(mask)
    a_o = o.alpha()
    n = mesh.n_nodes
    y_o = np.concatenate([o.system_matvec(a_o, x[:n]), o.system_matvec(a_o, x[n:])])
    assert rel(gff.system_matvec(x), y_o) < 1e-11, rel(gff.system_matvec(x), y_o)
    assert rel(gff.rhs(tmp), o.rhs(a_o, tmp)) < 1e-11
    p1, q1, s1 = gff.solve(tmp)
    p2, q2, s2 = g64.solve(tmp)
    assert s1["relative_residual"] <= 1e-11
    u1, u2 = np.where(mask == 1, q1, p1), np.where(mask == 1, q2, p2)
    assert rel(u1, u2) < 1e-9
    gff.close()
    g64.close()
