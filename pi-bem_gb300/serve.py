"""Request loop for many meshes on one GPU.

`BEMServer` answers solve requests (a mesh id and 1..n right-hand sides of
`tmp_rhs` data) with the FMM-GMRES solve of `pibem.BEMSolver`.  It keeps the
meshes it has seen resident on the device -- octree, near field, P2M/L2P tables
and Krylov space of one handle per mesh -- inside an HBM budget, evicting the
least recently used idle mesh when a new one would not fit.

Requests are taken in arrival order.  A worker that takes a request also takes
every request for the same mesh that is waiting at that moment (up to
`max_batch_rhs` columns) and solves them as one multi-RHS solve (continuous
batching): the operator applications are shared, the arithmetic of each column
is not, so every request gets the solution it would get alone.  Workers run on
their own threads; each handle owns a CUDA stream, so solves of different
meshes overlap on the GPU.  A handle is used by one worker at a time.

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
        self.batch_rhs = 0
        self.error = None
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
    max_batch_rhs   most columns of one coalesced solve
    solver_factory  callable(**params) -> solver with set_mesh / set_bc / solve /
                    device_bytes / close (default pibem.BEMSolver)
    defaults        pibem_params fields applied to every mesh (per-mesh fields
                    given to add_mesh override them)
    """

    def __init__(self, hbm_budget_gb: float = 150.0, workers: int = 4, max_batch_rhs: int = 16,
                 solver_factory=None, start: bool = True, **defaults):
        self.budget = float(hbm_budget_gb) * 1e9
        self.max_batch_rhs = int(max_batch_rhs)
        self.defaults = dict(defaults)
        self._factory = solver_factory or pibem.BEMSolver
        self._cv = threading.Condition()
        self._meshes: dict = {}
        self._pending: collections.deque = collections.deque()
        self._resident = 0
        self._next_id = 0
        self._stop = False
        self.counters = dict(setups=0, evictions=0, solves=0, columns=0, batches=0)
        self._threads = [threading.Thread(target=self._worker, name=f"pibem-serve-{i}", daemon=True)
                         for i in range(int(workers))]
        self._started = False
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

    def _take_batch(self):
        """Oldest waiting request whose mesh is free, plus the mesh's other
        waiting requests (arrival order, <= max_batch_rhs columns)."""
        for r in self._pending:
            m = self._meshes[r.mesh_id]
            if m.busy:
                continue
            batch, cols = [], 0
            for q in list(self._pending):
                if q.mesh_id != r.mesh_id:
                    continue
                if batch and cols + q.nrhs > self.max_batch_rhs:
                    break
                batch.append(q)
                cols += q.nrhs
            for q in batch:
                self._pending.remove(q)
            return m, batch
        return None, None

    def _worker(self):
        while True:
            with self._cv:
                while True:
                    if self._stop:
                        return
                    m, batch = self._take_batch()
                    if m is not None:
                        break
                    self._cv.wait()
                m.busy = True
                err = None
                try:
                    need = self._reserve(m)
                except Exception as e:  # budget or shutdown
                    need, err = False, e
            t0 = time.perf_counter()
            try:
                if err is not None:
                    raise err
                if need:
                    self._setup(m)
                self._solve(m, batch, t0)
            except Exception as e:
                for q in batch:
                    q.error = e
                    q.start = t0
                    q.end = time.perf_counter()
                    q._done.set()
            finally:
                with self._cv:
                    if m.handle is not None:
                        grown = int(m.handle.device_bytes())
                        self._resident += grown - m.bytes
                        m.bytes = grown
                    m.busy = False
                    m.last_used = time.perf_counter()
                    self._cv.notify_all()

    def _solve(self, m: _Mesh, batch, t0):
        tmp = np.concatenate([q.tmp for q in batch], axis=0)
        phi, dphi, st = m.handle.solve(tmp.reshape(-1))
        phi = phi.reshape(tmp.shape)
        dphi = dphi.reshape(tmp.shape)
        t1 = time.perf_counter()
        c = 0
        for q in batch:
            q.phi = phi[c:c + q.nrhs].copy()
            q.dphi_dn = dphi[c:c + q.nrhs].copy()
            q.stats = st
            q.batch_rhs = tmp.shape[0]
            q.start = t0
            q.end = t1
            c += q.nrhs
            q._done.set()
        with self._cv:
            self.counters["solves"] += len(batch)
            self.counters["columns"] += tmp.shape[0]
            self.counters["batches"] += 1
