"""Request loop for many meshes on one GPU.

`BEMServer` answers solve requests (a mesh id and 1..n right-hand sides of
`tmp_rhs` data) with the FMM-GMRES solve of `pibem.BEMSolver`.  It keeps the
meshes it has seen resident on the device -- octree, near field, P2M/L2P tables
and the Krylov spaces of one handle per mesh -- inside an HBM budget, evicting
the least recently used idle mesh when a new one would not fit.

Continuous batching: a worker serving a mesh keeps its handle's request slots
(`pibem_slots_*`, `max_batch_rhs` of them) busy.  Between steps of the solve
engine it admits the waiting requests of that mesh, oldest first, into free
slots (a request's columns may be admitted as slots free up); a column that
joins shares every operator application with the columns already in flight
from its next step on, and leaves as soon as it has converged, while the
others go on.  While slots are free, a step returns after at most
`quantum_steps` Arnoldi steps (or as soon as a column ends its GMRES cycle),
so that a request arriving in the middle of other requests' solves starts
within a few milliseconds.  A mesh admits new requests only while no older
request of another mesh is waiting for a worker (all workers busy): the
worker then finishes what it has in flight and moves on in arrival order.  Every column's
arithmetic is independent of the others', so each request gets the solution
it would get alone.  Workers run on their own threads; each handle owns a CUDA
stream, so different meshes overlap on the GPU.  A handle is served by one
worker at a time.

The reference solves one mesh per process (BEMProblem::solve,
source/bem_problem.cc:1352-1374); this loop is the serving layer around that
call and has no counterpart there.
"""
from __future__ import annotations

import collections
import threading
import time

import numpy as np

import pibem

__all__ = ["BEMServer", "Request", "estimate_bytes"]


def estimate_bytes(n_nodes: int, nrhs: int = 1, restart: int = 100) -> int:
    """Device bytes a handle is expected to hold for an n-node mesh, before it is
    set up (the near field dominates: a few hundred entries per row in five
    8-byte matrices (N, D, S and the two float-float pair matrices of the
    FP64-accurate operator) and one FP32 matrix; P2M and L2P tables; Krylov
    basis (restart + 1) x N per RHS).  The measured size (pibem_device_bytes)
    replaces it once the mesh is resident."""
    return int(n_nodes * (36_000 + 8 * (restart + 8) * max(1, nrhs)) + 64 * 2**20)


class Request:
    """One solve request: `tmp` holds `nrhs` columns of tmp_rhs (shape (nrhs, N))."""

    def __init__(self, rid: int, mesh_id, tmp: np.ndarray, arrival: float):
        self.rid = rid
        self.mesh_id = mesh_id
        self.tmp = tmp
        self.nrhs = tmp.shape[0]
        self.arrival = arrival
        self.start = None
        self.end = None
        self.phi = None
        self.dphi_dn = None
        self.stats = None
        self.batch_rhs = 0      # most columns in flight with this request's columns
        self.error = None
        self._next = 0          # columns admitted so far
        self._ndone = 0         # columns finished
        self._col_stats = []
        self._done = threading.Event()

    def wait(self, timeout: float | None = None) -> bool:
        return self._done.wait(timeout)

    @property
    def done(self) -> bool:
        return self._done.is_set()

    @property
    def latency(self) -> float:
        return self.end - self.arrival


class _Mesh:
    def __init__(self, mesh_id, xyz, cells, mask, params: dict, est: int):
        self.mesh_id = mesh_id
        self.xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        self.cells = np.ascontiguousarray(cells, np.int32).reshape(-1, 4)
        self.mask = np.ascontiguousarray(mask, np.uint8)
        self.params = params
        self.est = est
        self.handle = None
        self.bytes = 0     # bytes accounted for this mesh (estimate while setting up)
        self.busy = False
        self.last_used = 0.0

    @property
    def n(self) -> int:
        return self.xyz.shape[0]


class BEMServer:
    """Serve FMM-BEM solves for a set of registered meshes (see module docstring).

    hbm_budget_gb   device memory the resident meshes may hold together
    workers         threads issuing solves (each on its mesh's own stream)
    max_batch_rhs   request slots per mesh (columns in flight together)
    quantum_steps   Arnoldi steps per engine step while slots are free
    join_in_flight  admit a mesh's waiting requests while its solves are in
                    flight (False: only when the mesh has nothing in flight, the
                    waiting requests of the mesh then start together)
    solver_factory  callable(**params) -> solver with set_mesh / set_bc /
                    slots_open / slots_submit / slots_step / slots_collect /
                    device_bytes / close (default pibem.BEMSolver)
    defaults        pibem_params fields applied to every mesh (per-mesh fields
                    given to add_mesh override them)
    """

    def __init__(self, hbm_budget_gb: float = 150.0, workers: int = 4, max_batch_rhs: int = 16,
                 solver_factory=None, start: bool = True, quantum_steps: int = 16,
                 join_in_flight: bool = True, **defaults):
        self.budget = float(hbm_budget_gb) * 1e9
        self.max_batch_rhs = int(max_batch_rhs)
        self.quantum_steps = int(quantum_steps)
        self.join_in_flight = bool(join_in_flight)
        self.defaults = dict(defaults)
        self._factory = solver_factory or pibem.BEMSolver
        self._cv = threading.Condition()
        self._meshes: dict = {}
        self._pending: collections.deque = collections.deque()
        self._resident = 0
        self._next_id = 0
        self._stop = False
        self.counters = dict(setups=0, evictions=0, solves=0, columns=0, steps=0, admissions=0,
                             joined_in_flight=0)
        self._threads = [threading.Thread(target=self._worker, name=f"pibem-serve-{i}", daemon=True)
                         for i in range(int(workers))]
        self._started = False
        self._idle = 0   # workers waiting for work
        if start:
            self.start()

    # -- public -------------------------------------------------------------
    def start(self):
        if not self._started:
            self._started = True
            for t in self._threads:
                t.start()

    def add_mesh(self, mesh_id, xyz, cells, dirichlet_mask, est_bytes: int | None = None,
                 **params):
        p = dict(self.defaults)
        p.update(params)
        n = np.asarray(xyz).reshape(-1, 3).shape[0]
        est = est_bytes if est_bytes is not None else estimate_bytes(
            n, self.max_batch_rhs, p.get("gmres_restart", 100))
        with self._cv:
            if mesh_id in self._meshes:
                raise KeyError(f"mesh {mesh_id!r} already registered")
            self._meshes[mesh_id] = _Mesh(mesh_id, xyz, cells, dirichlet_mask, p, est)

    def preload(self, mesh_id):
        """Set the mesh up on the device now (blocking), within the budget."""
        m = self._meshes[mesh_id]
        with self._cv:
            while m.busy:
                self._cv.wait()
            m.busy = True
            try:
                need = self._reserve(m)
            except Exception:
                m.busy = False
                self._cv.notify_all()
                raise
        try:
            if need:
                self._setup(m)
        finally:
            with self._cv:
                m.busy = False
                m.last_used = time.perf_counter()
                self._cv.notify_all()

    def submit(self, mesh_id, tmp_rhs, arrival: float | None = None) -> Request:
        """Queue a request; tmp_rhs has shape (N,) or (nrhs, N)."""
        m = self._meshes[mesh_id]
        t = np.ascontiguousarray(tmp_rhs, np.float64).reshape(-1, m.n)
        with self._cv:
            if self._stop:
                raise RuntimeError("server is closed")
            r = Request(self._next_id, mesh_id, t, time.perf_counter() if arrival is None else arrival)
            self._next_id += 1
            self._pending.append(r)
            self._cv.notify_all()
        return r

    def resident_bytes(self) -> int:
        with self._cv:
            return self._resident

    def resident_meshes(self) -> list:
        with self._cv:
            return [k for k, m in self._meshes.items() if m.handle is not None]

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            if t.is_alive():
                t.join()
        with self._cv:
            for m in self._meshes.values():
                if m.handle is not None:
                    m.handle.close()
                    m.handle = None
                    self._resident -= m.bytes
                    m.bytes = 0
            for r in self._pending:
                r.error = RuntimeError("server closed")
                r._done.set()
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- internals (call with self._cv held unless noted) -----------------------
    def _reserve(self, m: _Mesh) -> bool:
        """Make room for m (evicting idle meshes); True if m must be set up."""
        if m.handle is not None:
            return False
        if m.est > self.budget:
            raise MemoryError(f"mesh {m.mesh_id!r} needs ~{m.est / 1e9:.1f} GB, more than the "
                              f"{self.budget / 1e9:.1f} GB budget")
        while self._resident + m.est > self.budget:
            idle = [x for x in self._meshes.values()
                    if x.handle is not None and not x.busy and x is not m]
            if idle:
                v = min(idle, key=lambda x: x.last_used)
                v.handle.close()
                v.handle = None
                self._resident -= v.bytes
                v.bytes = 0
                self.counters["evictions"] += 1
                continue
            if self._stop:
                raise RuntimeError("server closed")
            self._cv.wait()   # a busy mesh will become idle
        self._resident += m.est
        m.bytes = m.est
        return True

    def _setup(self, m: _Mesh):
        """Create the handle (no lock held)."""
        try:
            h = self._factory(**m.params)
            h.set_mesh(m.xyz, m.cells)
            h.set_bc(m.mask)
            h.slots_open(self.max_batch_rhs)
            actual = int(h.device_bytes())
        except Exception:
            with self._cv:
                self._resident -= m.bytes
                m.bytes = 0
            raise
        with self._cv:
            m.handle = h
            self._resident += actual - m.bytes
            m.bytes = actual
            self.counters["setups"] += 1

    def _next_mesh(self):
        """Mesh of the oldest waiting request that no worker is serving."""
        for r in self._pending:
            m = self._meshes[r.mesh_id]
            if not m.busy:
                return m
        return None

    def _worker(self):
        while True:
            with self._cv:
                while True:
                    if self._stop:
                        return
                    m = self._next_mesh()
                    if m is not None:
                        break
                    self._idle += 1
                    self._cv.wait()
                    self._idle -= 1
                m.busy = True
                err = None
                try:
                    need = self._reserve(m)
                except Exception as e:  # budget or shutdown
                    need, err = False, e
            flight = {}
            try:
                if err is not None:
                    raise err
                if need:
                    self._setup(m)
                self._serve(m, flight)
            except Exception as e:
                t = time.perf_counter()
                with self._cv:
                    # the mesh's requests in flight and, if the mesh failed
                    # before serving, its waiting ones
                    failed = list(flight)
                    if not flight:
                        failed = [q for q in self._pending if q.mesh_id == m.mesh_id]
                        for q in failed:
                            self._pending.remove(q)
                for q in failed:
                    q.error = e
                    q.start = q.start if q.start is not None else t
                    q.end = t
                    q._done.set()
                if m.handle is not None and flight:
                    # the slots' state is unknown after a failure: a fresh set
                    try:
                        m.handle.slots_close()
                        m.handle.slots_open(self.max_batch_rhs)
                    except Exception:
                        pass
            finally:
                with self._cv:
                    if m.handle is not None:
                        grown = int(m.handle.device_bytes())
                        self._resident += grown - m.bytes
                        m.bytes = grown
                    m.busy = False
                    m.last_used = time.perf_counter()
                    self._cv.notify_all()

    def _serve(self, m: _Mesh, flight: dict):
        """Keep the mesh's slots busy until no request of it is in flight or
        waiting (no lock held)."""
        h = m.handle
        cap = self.max_batch_rhs
        cols = {}      # column id -> (request, column)
        used = 0
        cid = 0
        while True:
            admitted = []
            with self._cv:
                for q in list(self._pending):
                    if q.mesh_id != m.mesh_id:
                        # an older request of a mesh no worker serves, and no
                        # idle worker to take it: this mesh admits nothing
                        # newer until its work in flight is done (the worker then
                        # moves on in arrival order)
                        if not self._meshes[q.mesh_id].busy and self._idle == 0:
                            break
                        continue
                    if used >= cap or (flight and not self.join_in_flight and q not in flight):
                        break
                    k = min(q.nrhs - q._next, cap - used)
                    admitted.append((q, q._next, k))
                    q._next += k
                    used += k
                    if q._next == q.nrhs:
                        self._pending.remove(q)
                    else:
                        break  # arrival order: the rest of q before any later request
                if admitted:
                    self.counters["admissions"] += 1
                    if flight:
                        self.counters["joined_in_flight"] += 1
                # requests of this mesh still waiting (slots full, or held
                # back): only then does a step return early to admit them
                waiting = any(q.mesh_id == m.mesh_id for q in self._pending)
            if not flight and not admitted:
                return
            t = time.perf_counter()
            for q, c0, k in admitted:
                if q not in flight:
                    flight[q] = True
                    q.start = t
                    q.phi = np.empty_like(q.tmp)
                    q.dphi_dn = np.empty_like(q.tmp)
                    q._col_stats = [None] * q.nrhs
                for c in range(c0, c0 + k):
                    cols[cid] = (q, c)
                    if h.slots_submit(cid, q.tmp[c]) is None:
                        raise RuntimeError("no free request slot")
                    cid += 1
            for q in flight:
                q.batch_rhs = max(q.batch_rhs, used)
            # with nobody waiting the step runs until every column has ended its
            # GMRES cycle, so that the columns' FP64-accurate residuals and
            # corrections are taken together (one operator application for all)
            h.slots_step(self.quantum_steps if (used < cap and waiting) else 0)
            with self._cv:
                self.counters["steps"] += 1
            while True:
                res = h.slots_collect()
                if res is None:
                    break
                rid, phi, dphi, st = res
                q, c = cols.pop(rid)
                used -= 1
                q.phi[c] = phi
                q.dphi_dn[c] = dphi
                q._col_stats[c] = st
                q._ndone += 1
                if not st.get("converged", True) and q.error is None:
                    q.error = pibem.PibemError(pibem.ENOCONV, "request did not reach the tolerance")
                if q._ndone == q.nrhs:
                    q.end = time.perf_counter()
                    q.stats = _merge_stats(q._col_stats)
                    flight.pop(q)
                    with self._cv:
                        self.counters["solves"] += 1
                        self.counters["columns"] += q.nrhs
                    q._done.set()


def _merge_stats(cols):
    """A request's statistics from its columns': the worst residual, the most
    iterations and refinement steps, the operator applications summed."""
    out = {"iterations": max(c["iterations"] for c in cols),
           "refinement_steps": max(c["refinement_steps"] for c in cols),
           "fp64_matvecs": sum(c["fp64_matvecs"] for c in cols),
           "fp32_matvecs": sum(c["fp32_matvecs"] for c in cols),
           "relative_residual": max(c["relative_residual"] for c in cols),
           "seconds": max(c["seconds"] for c in cols)}
    return out
