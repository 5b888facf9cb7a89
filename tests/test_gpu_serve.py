"""The request loop on the GPU: requests coalesced into one multi-RHS solve get
exactly the solution each gets alone (bitwise), in both precision modes, and
meshes evicted under a small HBM budget come back with the same results."""
import numpy as np
import pytest

import serve

pytestmark = pytest.mark.gpu


def _cases(S):
    out = {}
    m = S.perturbed_sphere(10, seed=21)
    out["sphere"] = (m, S.random_plane_mask(m, 22), "ball")
    m = S.wigley_hull(*S.wigley_for_nodes(3000))
    out["wigley"] = (m, S.random_plane_mask(m, 23), "wigley")
    return out


def _rhs(S, mesh, mask, where, seed, nrhs):
    rng = np.random.Generator(np.random.PCG64(seed))
    cols = []
    for _ in range(nrhs):
        src = S.sources_in_ball(rng, 4) if where == "ball" else S.sources_in_wigley(rng, 4)
        cols.append(S.point_source_data(mesh, mask, src, rng.uniform(-1, 1, 4))[0])
    return np.stack(cols)


PARAMS = dict(fma_truncation_order=6, max_nodes_per_childless_block=20, is_external_flow=1)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_coalesced_requests_equal_alone(mode, pibem_mod, synthetic):
    S = synthetic
    prm = dict(PARAMS, precision_mode=pibem_mod.PRECISION_MIXED if mode == "mixed"
               else pibem_mod.PRECISION_FP64)
    cases = _cases(S)
    srv = serve.BEMServer(hbm_budget_gb=20, workers=2, max_batch_rhs=16, start=False, **prm)
    reqs = []
    for k, (mesh, mask, where) in cases.items():
        srv.add_mesh(k, mesh.xyz, mesh.cells, mask)
        for i, R in enumerate((1, 3, 2)):
            reqs.append((k, srv.submit(k, _rhs(S, mesh, mask, where, 100 + i, R))))
    srv.start()
    for _, r in reqs:
        assert r.wait(600) and r.error is None, r.error
        assert r.batch_rhs == 6
    srv.close()
    for k, r in reqs:
        mesh, mask, _ = cases[k]
        g = pibem_mod.BEMSolver(**prm)
        g.set_mesh(mesh.xyz, mesh.cells)
        g.set_bc(mask)
        phi, dphi, st = g.solve(r.tmp.reshape(-1))
        g.close()
        assert st["relative_residual"] <= 1e-8
        np.testing.assert_array_equal(phi.reshape(r.tmp.shape), r.phi)
        np.testing.assert_array_equal(dphi.reshape(r.tmp.shape), r.dphi_dn)


def test_eviction_under_small_budget_keeps_results(pibem_mod, synthetic):
    S = synthetic
    cases = _cases(S)
    prm = dict(PARAMS, precision_mode=pibem_mod.PRECISION_MIXED)
    # measure the two meshes, then give the server room for only the larger one
    sizes = {}
    for k, (mesh, mask, _) in cases.items():
        g = pibem_mod.BEMSolver(**prm)
        g.set_mesh(mesh.xyz, mesh.cells)
        g.set_bc(mask)
        g.solve(np.ones(mesh.n_nodes))
        sizes[k] = g.device_bytes()
        g.close()
    budget = max(sizes.values()) + 0.5 * min(sizes.values())  # never both at once
    srv = serve.BEMServer(hbm_budget_gb=budget / 1e9, workers=1, max_batch_rhs=1, **prm)
    for k, (mesh, mask, _) in cases.items():
        srv.add_mesh(k, mesh.xyz, mesh.cells, mask, est_bytes=sizes[k])
    first = {}
    for rep in range(2):
        for k, (mesh, mask, where) in cases.items():
            r = srv.submit(k, _rhs(S, mesh, mask, where, 7, 1))
            assert r.wait(600) and r.error is None, r.error
            if rep == 0:
                first[k] = r.phi
            else:
                np.testing.assert_array_equal(first[k], r.phi)
            assert srv.resident_bytes() <= budget
    assert srv.counters["evictions"] >= 3 and srv.counters["setups"] >= 4
    srv.close()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_slots_request_joining_mid_solve_equals_alone(mode, pibem_mod, synthetic):
    """Request slots (pibem_slots_*): a right-hand side submitted while another
    is in the middle of its GMRES cycle joins the batch at the next step (a few
    Arnoldi steps per engine step) and both results are bitwise those of
    pibem_solve alone, with their own statistics."""
    S = synthetic
    prm = dict(PARAMS, precision_mode=pibem_mod.PRECISION_MIXED if mode == "mixed"
               else pibem_mod.PRECISION_FP64)
    mesh, mask, where = _cases(S)["wigley"]
    ta = _rhs(S, mesh, mask, where, 41, 1)[0]
    tb = _rhs(S, mesh, mask, where, 42, 1)[0]
    g = pibem_mod.BEMSolver(**prm)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    alone = {k: g.solve(t) for k, t in (("a", ta), ("b", tb))}
    g.slots_open(4)
    assert g.slots_submit(7, ta) is not None
    steps_before_b = 0
    for _ in range(3):
        act, done = g.slots_step(max_steps=2)
        steps_before_b += 1
        assert act == 1 and done == 0  # a is still in flight
    assert g.slots_submit(3, tb) is not None
    got = {}
    for _ in range(10000):
        act, done = g.slots_step(max_steps=2)
        while True:
            res = g.slots_collect()
            if res is None:
                break
            got[res[0]] = res
        if len(got) == 2:
            break
    assert sorted(got) == [3, 7]
    for rid, key in ((7, "a"), (3, "b")):
        _, phi, dphi, st = got[rid]
        p0, d0, s0 = alone[key]
        np.testing.assert_array_equal(phi, p0)
        np.testing.assert_array_equal(dphi, d0)
        assert st["converged"] and st["relative_residual"] == s0["relative_residual"]
        assert st["iterations"] == s0["iterations"]
    # the solve entry point is refused while slots are open
    with pytest.raises(pibem_mod.PibemError):
        g.solve(ta)
    g.slots_close()
    g.close()
