"""The FP32 operator replayed as a CUDA graph gives bitwise the same results as
its direct launch sequence (phase timing on disables the graph), for operator
applications and whole mixed-precision solves, and the library's launch
counter counts the graph's kernels at every replay."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle(pibem, S, p=6):
    mesh, mask, tmp, _, _ = S.spheroid_mixed_case(14, seed=2)
    g = pibem.BEMSolver(fma_truncation_order=p, max_nodes_per_childless_block=20,
                        is_external_flow=1, precision_mode=pibem.PRECISION_MIXED)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    return g, mesh, tmp


def test_graph_matches_direct_launches(pibem_mod, synthetic):
    g, mesh, tmp = _handle(pibem_mod, synthetic)
    x = np.random.Generator(np.random.PCG64(3)).normal(size=(2, mesh.n_nodes))
    os.environ["PIBEM_MATVEC_FP32"] = "1"
    try:
        g.set_profiling(True)   # direct launches
        y_direct = g.system_matvec(x.reshape(-1))
        l0 = pibem_mod.launch_count()
        g.system_matvec(x.reshape(-1))
        per_direct = pibem_mod.launch_count() - l0
        g.set_profiling(False)  # first call captures, later calls replay
        y_first = g.system_matvec(x.reshape(-1))
        l0 = pibem_mod.launch_count()
        y_replay = g.system_matvec(x.reshape(-1))
        per_call = pibem_mod.launch_count() - l0
    finally:
        os.environ.pop("PIBEM_MATVEC_FP32", None)
    np.testing.assert_array_equal(y_direct, y_first)
    np.testing.assert_array_equal(y_direct, y_replay)
    assert per_call == per_direct > 5  # the graph's kernels are counted at replay
    g.set_profiling(True)
    p1, d1, s1 = g.solve(tmp)
    g.set_profiling(False)
    p2, d2, s2 = g.solve(tmp)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(d1, d2)
    assert s1["iterations"] == s2["iterations"] and s2["relative_residual"] <= 1e-8
    g.close()


def test_graph_is_rebuilt_after_new_mesh(pibem_mod, synthetic):
    S = synthetic
    g, mesh, tmp = _handle(pibem_mod, S)
    g.solve(tmp)
    m2, mask2, tmp2, _, _ = S.spheroid_mixed_case(10, seed=5)
    g.set_mesh(m2.xyz, m2.cells)
    g.set_bc(mask2)
    ph, dp, st = g.solve(tmp2)
    ref = pibem_mod.BEMSolver(fma_truncation_order=6, max_nodes_per_childless_block=20,
                              is_external_flow=1, precision_mode=pibem_mod.PRECISION_MIXED)
    ref.set_mesh(m2.xyz, m2.cells)
    ref.set_bc(mask2)
    ph2, dp2, _ = ref.solve(tmp2)
    np.testing.assert_array_equal(ph, ph2)
    np.testing.assert_array_equal(dp, dp2)
    g.close()
    ref.close()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_gmres_cycle_graph_matches_step_launches(pibem_mod, synthetic, mode):
    """A GMRES restart cycle runs as one CUDA graph (a conditional while node
    around one Arnoldi step, with the Givens rotation and the stopping test on
    the device); with phase timing on (with and without the hold kernel before
    each operator application) the same launches are issued step by step.
    Solutions, iteration counts, operator counts and launch counts agree, for
    one column and for a batch of three."""
    S = synthetic
    mesh, mask, tmp, _, _ = S.spheroid_mixed_case(14, seed=2)
    prec = pibem_mod.PRECISION_FP64 if mode == "fp64" else pibem_mod.PRECISION_MIXED
    g = pibem_mod.BEMSolver(fma_truncation_order=6, max_nodes_per_childless_block=20,
                            is_external_flow=1, precision_mode=prec, gmres_restart=8)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    for t in (tmp, np.stack([tmp, 0.5 * tmp + 0.1, -tmp])):
        out = []
        for prof in (True, 2, False, False):
            g.set_profiling(prof)
            l0 = pibem_mod.launch_count()
            p, d, st = g.solve(t)
            out.append((p, d, st, pibem_mod.launch_count() - l0))
        for p, d, st, nl in out[1:]:
            np.testing.assert_array_equal(p, out[0][0])
            np.testing.assert_array_equal(d, out[0][1])
            for k in ("iterations", "fp32_matvecs", "fp64_matvecs", "refinement_steps"):
                assert st[k] == out[0][2][k], k
            assert nl == out[0][3]
        assert out[0][2]["relative_residual"] <= 1e-8
        # restarts (restart length 8) happened on the way
        assert out[0][2]["iterations"] > 8
    g.set_profiling(False)
    g.close()
