"""Host logic of the request loop (pi-bem_gb300/serve.py) with a fake solver:
admission of waiting requests per mesh into the request slots, the slot cap,
requests joining a batch in flight (continuous batching), LRU eviction under
the HBM budget, refusal of a mesh larger than the budget, error propagation and
overlap of different meshes on different workers.  No GPU."""
import threading
import time

import numpy as np
import pytest

import serve


class FakeSolver:
    """Stands in for pibem.BEMSolver's request slots: phi = 2 tmp, dphi = -tmp;
    a column finishes after `steps` engine steps (each takes `delay` seconds).
    Every step is logged as (solver, columns in flight, start, end)."""
    log = []
    lock = threading.Lock()

    def __init__(self, fake_bytes=10**9, delay=0.0, fail=False, steps=1, **_):
        self.bytes = fake_bytes
        self.delay = delay
        self.fail = fail
        self.steps = steps
        self.closed = False
        self.cap = 0
        self.cols = {}   # rid -> [tmp, steps left]
        self.done = {}

    def set_mesh(self, xyz, cells):
        self.n = np.asarray(xyz).reshape(-1, 3).shape[0]

    def set_bc(self, mask):
        self.mask = mask

    def device_bytes(self):
        return self.bytes

    def slots_open(self, cap):
        self.cap = cap
        self.cols.clear()
        self.done.clear()

    def slots_close(self):
        self.cap = 0

    def slots_submit(self, rid, tmp):
        if len(self.cols) + len(self.done) >= self.cap:
            return None
        self.cols[rid] = [np.array(tmp), self.steps]
        return len(self.cols) - 1

    def slots_step(self, max_steps=0):
        t0 = time.perf_counter()
        if self.delay:
            time.sleep(self.delay)
        if self.fail:
            raise RuntimeError("solver failed")
        with FakeSolver.lock:
            FakeSolver.log.append((id(self), len(self.cols), t0, time.perf_counter()))
        for rid in list(self.cols):
            self.cols[rid][1] -= 1
            if self.cols[rid][1] <= 0:
                self.done[rid] = self.cols.pop(rid)[0]
        return len(self.cols), len(self.done)

    def slots_collect(self):
        if not self.done:
            return None
        rid = min(self.done)
        t = self.done.pop(rid)
        return rid, 2 * t, -t, {"iterations": 1, "refinement_steps": 0, "fp64_matvecs": 1,
                                "fp32_matvecs": 0, "relative_residual": 0.0, "seconds": 0.0,
                                "converged": True}

    def close(self):
        self.closed = True


def _mesh(n=10):
    xyz = np.zeros((n, 3))
    cells = np.zeros((1, 4), np.int32)
    return xyz, cells, np.zeros(n, np.uint8)


@pytest.fixture(autouse=True)
def _clear_log():
    FakeSolver.log.clear()


def test_waiting_requests_for_one_mesh_are_coalesced():
    s = serve.BEMServer(hbm_budget_gb=100, workers=1, max_batch_rhs=16,
                        solver_factory=FakeSolver, start=False)
    for k in ("A", "B"):
        s.add_mesh(k, *_mesh())
    rng = np.random.default_rng(0)
    reqs = [s.submit("A", rng.normal(size=(r, 10))) for r in (1, 2, 3)]
    rb = s.submit("B", rng.normal(size=(2, 10)))
    s.start()
    for r in reqs + [rb]:
        assert r.wait(10) and r.error is None
    assert [r.batch_rhs for r in reqs] == [6, 6, 6] and rb.batch_rhs == 2
    for r in reqs + [rb]:
        np.testing.assert_array_equal(r.phi, 2 * r.tmp)
        np.testing.assert_array_equal(r.dphi_dn, -r.tmp)
    assert sorted(R for _, R, _, _ in FakeSolver.log) == [2, 6]
    assert s.counters["admissions"] == 2 and s.counters["columns"] == 8
    s.close()


def test_column_cap_splits_batches_in_arrival_order():
    s = serve.BEMServer(hbm_budget_gb=100, workers=1, max_batch_rhs=8,
                        solver_factory=FakeSolver, start=False)
    s.add_mesh("A", *_mesh())
    reqs = [s.submit("A", np.full((4, 10), float(i))) for i in range(5)]
    s.start()
    for r in reqs:
        assert r.wait(10)
    assert [r.batch_rhs for r in reqs] == [8, 8, 8, 8, 4]
    assert [R for _, R, _, _ in FakeSolver.log] == [8, 8, 4]
    s.close()


def test_lru_eviction_keeps_resident_bytes_within_budget():
    s = serve.BEMServer(hbm_budget_gb=10, workers=1, solver_factory=FakeSolver)
    for k in "ABC":
        s.add_mesh(k, *_mesh(), est_bytes=4 * 10**9, fake_bytes=4 * 10**9)
    for k in "AB":
        assert s.submit(k, np.ones(10)).wait(10)
    assert sorted(s.resident_meshes()) == ["A", "B"]
    assert s.submit("A", np.ones(10)).wait(10)  # A is now the most recently used
    r = s.submit("C", np.ones(10))
    assert r.wait(10) and r.error is None
    assert sorted(s.resident_meshes()) == ["A", "C"]  # B was least recently used
    assert s.counters["evictions"] == 1 and s.resident_bytes() <= 10 * 10**9
    s.close()
    assert s.resident_bytes() == 0


def test_mesh_larger_than_budget_is_refused_and_server_continues():
    s = serve.BEMServer(hbm_budget_gb=1, workers=1, solver_factory=FakeSolver)
    s.add_mesh("big", *_mesh(), est_bytes=5 * 10**9)
    s.add_mesh("ok", *_mesh(), est_bytes=10**8, fake_bytes=10**8)
    r = s.submit("big", np.ones(10))
    assert r.wait(10) and isinstance(r.error, MemoryError)
    r2 = s.submit("ok", np.ones(10))
    assert r2.wait(10) and r2.error is None
    s.close()


def test_solver_error_reaches_the_request():
    s = serve.BEMServer(hbm_budget_gb=100, workers=1, solver_factory=FakeSolver)
    s.add_mesh("bad", *_mesh(), fail=True)
    s.add_mesh("good", *_mesh())
    r = s.submit("bad", np.ones(10))
    assert r.wait(10) and isinstance(r.error, RuntimeError)
    r2 = s.submit("good", np.ones(10))
    assert r2.wait(10) and r2.error is None
    s.close()


def test_request_arriving_mid_solve_joins_the_batch_in_flight():
    """A request submitted while another of the same mesh is in flight starts
    before that one ends (it joins at the next engine step) and gets its own
    result."""
    s = serve.BEMServer(hbm_budget_gb=100, workers=1, solver_factory=FakeSolver)
    s.add_mesh("A", *_mesh(), delay=0.05, steps=6)
    s.preload("A")
    ra = s.submit("A", np.full((1, 10), 1.0))
    while ra.start is None:
        time.sleep(0.005)
    time.sleep(0.08)  # ra is a step or two into its solve
    rb = s.submit("A", np.full((2, 10), 3.0))
    assert ra.wait(10) and rb.wait(10) and ra.error is None and rb.error is None
    assert rb.start < ra.end and ra.start < rb.start
    assert ra.batch_rhs == 3 and rb.batch_rhs == 3
    assert s.counters["joined_in_flight"] == 1
    np.testing.assert_array_equal(rb.phi, 2 * rb.tmp)
    s.close()


def test_different_meshes_overlap_on_two_workers():
    s = serve.BEMServer(hbm_budget_gb=100, workers=2, solver_factory=FakeSolver, start=False)
    for k in "AB":
        s.add_mesh(k, *_mesh(), delay=0.3)
        s.preload(k)
    ra, rb = s.submit("A", np.ones(10)), s.submit("B", np.ones(10))
    s.start()
    assert ra.wait(10) and rb.wait(10)
    (_, _, a0, a1), (_, _, b0, b1) = FakeSolver.log
    assert max(a0, b0) < min(a1, b1)  # the two solves ran at the same time
    assert s.counters["setups"] == 2
    s.close()


def test_estimate_grows_with_nodes_and_columns():
    assert serve.estimate_bytes(2000) < serve.estimate_bytes(200_000)
    assert serve.estimate_bytes(10_000, 1) < serve.estimate_bytes(10_000, 16)
