"""The fused level passes of the FP32 operator (levels.cu: M2M summed into the
parents and L2L added to the M2L sums, one launch per level) against the
batched-GEMM + gather level passes, which the operator takes for more than 16
right-hand sides, and against the FP64 operator.

Tolerances: the two FP32 level implementations agree to 2e-6 relative
(2-norm), the FP32 operator is within 2e-5 of the FP64 operator.  A column's
result through the fused passes does not depend on the other columns: the
same bits alone and in batches of 3 and 16."""
import os

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

CASES = [
    ("spheroid_p8", dict(n=20, p=8, leaf=40)),
    ("spheroid_p6_deep", dict(n=24, p=6, leaf=8)),
    ("spheroid_p10", dict(n=16, p=10, leaf=30)),
]


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
def test_fused_levels(name, c, pibem_mod, synthetic):
    mesh, mask = synthetic.spheroid_mixed_case(c["n"], seed=2)[:2]
    n = mesh.n_nodes
    rng = np.random.Generator(np.random.PCG64(9))
    X = rng.normal(size=(17, n))
    prm = dict(fma_truncation_order=c["p"], max_nodes_per_childless_block=c["leaf"],
               is_external_flow=1)
    g = pibem_mod.BEMSolver(precision_mode=pibem_mod.PRECISION_MIXED, **prm)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    os.environ["PIBEM_MATVEC_FP32"] = "1"
    try:
        y1 = np.stack([g.system_matvec(X[i]) for i in range(3)])
        y3 = g.system_matvec(X[:3].reshape(-1)).reshape(3, n)
        y16 = g.system_matvec(X[:16].reshape(-1)).reshape(16, n)
        y17 = g.system_matvec(X.reshape(-1)).reshape(17, n)  # GEMM + gather levels
    finally:
        os.environ.pop("PIBEM_MATVEC_FP32", None)
    np.testing.assert_array_equal(y1, y3)
    np.testing.assert_array_equal(y1, y16[:3])
    g64 = pibem_mod.BEMSolver(precision_mode=pibem_mod.PRECISION_FP64, **prm)
    g64.set_mesh(mesh.xyz, mesh.cells)
    g64.set_bc(mask)
    y64 = g64.system_matvec(X[:3].reshape(-1)).reshape(3, n)
    for i in range(3):
        assert rel(y1[i], y17[i]) < 2e-6, rel(y1[i], y17[i])
        assert rel(y1[i], y64[i]) < 2e-5, rel(y1[i], y64[i])
    g.close()
    g64.close()
