"""The tensor-core (tcgen05, 3xTF32) translation GEMM of the FP32 operator
against the CUDA-core FP32 GEMM, the FP64 operator and the oracle's operator
(BEMProblem::vmult restated on the CPU), through the C ABI.

Tolerance: both FP32 operators agree to 2e-6 relative (2-norm); the FP32
operator is within 2e-5 of the FP64 operator and of the oracle."""
import os

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

CASES = [
    ("sphere_p4", dict(n=12, p=4, leaf=30, ext=False)),
    ("perturbed_p6", dict(n=14, p=6, leaf=12, ext=True, perturbed=True)),
    ("spheroid_p8", dict(n=20, p=8, leaf=40, ext=True)),
    ("spheroid_p10", dict(n=16, p=10, leaf=30, ext=True)),
]


def _mesh(S, c):
    if c.get("perturbed"):
        mesh = S.perturbed_sphere(c["n"], seed=11)
        return S.spheroid_mixed_case(0, seed=4, mesh=mesh)[:2]
    if c["ext"]:
        return S.spheroid_mixed_case(c["n"], seed=2)[:2]
    mesh, mask, _, _ = S.sphere_dirichlet_case(c["n"])
    return mesh, mask


def _handle(pibem, c, mesh, mask, mode, tc):
    g = pibem.BEMSolver(fma_truncation_order=c["p"], max_nodes_per_childless_block=c["leaf"],
                        is_external_flow=int(c["ext"]), precision_mode=mode,
                        m2l_engine=pibem.M2L_TENSOR_CORE if tc else pibem.M2L_CUDA_CORE)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    return g


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
def test_tensor_core_translations(name, c, pibem_mod, synthetic, oracle_mod):
    mesh, mask = _mesh(synthetic, c)
    x = np.random.Generator(np.random.PCG64(5)).normal(size=mesh.n_nodes)
    os.environ["PIBEM_MATVEC_FP32"] = "1"
    try:
        g_tc = _handle(pibem_mod, c, mesh, mask, pibem_mod.PRECISION_MIXED, True)
        g_cc = _handle(pibem_mod, c, mesh, mask, pibem_mod.PRECISION_MIXED, False)
        y_tc = g_tc.system_matvec(x)
        y_cc = g_cc.system_matvec(x)
    finally:
        os.environ.pop("PIBEM_MATVEC_FP32", None)
    g64 = _handle(pibem_mod, c, mesh, mask, pibem_mod.PRECISION_FP64, False)
    y64 = g64.system_matvec(x)
    assert rel(y_tc, y_cc) < 2e-6, rel(y_tc, y_cc)
    assert rel(y_tc, y64) < 2e-5, rel(y_tc, y64)
    o = oracle_mod.Oracle(p=c["p"], levels=10, max_nodes=c["leaf"], external=c["ext"])
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_bc(mask)
    y_o = o.system_matvec(o.alpha(), x)
    assert rel(y_tc, y_o) < 2e-5, rel(y_tc, y_o)
    # the solve through the tensor-core operator meets the FP64 residual
    tmp = np.where(mask == 1, 1.0, 0.5) * np.cos(mesh.xyz[:, 0])
    _, _, st = g_tc.solve(tmp)
    assert st["relative_residual"] <= 1e-8 and st["fp32_matvecs"] > 0
    for g in (g_tc, g_cc, g64):
        g.close()
