"""The fused level passes of the FP32 operator (levels.cu: M2M summed into the
parents, target-major M2L sums, L2L added to them, one launch per level)
against the FP64 operator, and the independence of a column's result from
the batch it is in.

Tolerance: the FP32 operator is within 2e-5 of the FP64 operator (2-norm, per
column).  A column's result does not depend on the other columns: the same
bits alone and in batches of 3, 16 and 17 columns."""
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
        y17 = g.system_matvec(X.reshape(-1)).reshape(17, n)
    finally:
        os.environ.pop("PIBEM_MATVEC_FP32", None)
    for yb in (y3, y16[:3], y17[:3]):
        np.testing.assert_array_equal(y1, yb)
    np.testing.assert_array_equal(y16, y17[:16])
    g64 = pibem_mod.BEMSolver(precision_mode=pibem_mod.PRECISION_FP64, **prm)
    g64.set_mesh(mesh.xyz, mesh.cells)
    g64.set_bc(mask)
    y64 = g64.system_matvec(X[:3].reshape(-1)).reshape(3, n)
    for i in range(3):
        assert rel(y1[i], y64[i]) < 2e-5, rel(y1[i], y64[i])
    g.close()
    g64.close()
