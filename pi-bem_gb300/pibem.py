"""ctypes binding of libpibem_gb300.so (include/pibem_gpu.h).

Mirrors the reference's BEMFMA / BEMProblem call surface:
    set_mesh      ~ BEMFMA::init_fma + generate_octree_blocking + direct_integrals
                    + multipole_integrals
    fmm_matvec    ~ generate_multipole_expansions + multipole_matr_vect_products
    alpha         ~ BEMProblem::compute_alpha
    system_matvec ~ BEMProblem::vmult
    rhs           ~ BEMProblem::compute_rhs
    solve         ~ BEMProblem::solve_system
Errors raise PibemError carrying the C status code and message.  There is no
fallback: if the CUDA library is missing or cannot be loaded, import fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpibem_gb300.so")

OK, EINVAL, ENOMEM_HBM, ENOCONV, ETIMEDOUT, ECUDA, EAGAIN = 0, 1, 2, 3, 4, 5, 6
PRECISION_FP64, PRECISION_MIXED, PRECISION_FLOAT_FLOAT = 0, 1, 2
M2L_TENSOR_CORE, M2L_CUDA_CORE = 0, 1
PREC_NONE, PREC_BLOCK_JACOBI, PREC_ILU = 0, 1, 2


class Params(C.Structure):
    _fields_ = [
        ("fma_truncation_order", C.c_int32),
        ("num_octree_levels", C.c_int32),
        ("max_nodes_per_childless_block", C.c_int32),
        ("quadrature_order", C.c_int32),
        ("singular_quadrature_order", C.c_int32),
        ("solver_max_steps", C.c_int32),
        ("solver_tolerance", C.c_double),
        ("gmres_restart", C.c_int32),
        ("is_external_flow", C.c_int32),
        ("precision_mode", C.c_int32),
        ("preconditioner", C.c_int32),
        ("device", C.c_int32),
        ("inner_tolerance", C.c_double),
        ("hbm_budget_gb", C.c_double),
        ("m2l_engine", C.c_int32),
        ("double_body", C.c_int32),
        ("symmetry_plane_z_level", C.c_double),
        ("continuous_gradient", C.c_int32),
        ("m2l_chunk_pairs", C.c_int32),
        ("m2l_stages", C.c_int32),
    ]


class SolveStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("refinement_steps", C.c_int32),
        ("fp64_matvecs", C.c_int32),
        ("fp32_matvecs", C.c_int32),
        ("relative_residual", C.c_double),
        ("seconds", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TreeInfo(C.Structure):
    _fields_ = [
        ("n_boxes", C.c_int32),
        ("n_levels", C.c_int32),
        ("n_leaves", C.c_int32),
        ("n_m2l_pairs", C.c_int64),
        ("n_m2p_pairs", C.c_int64),
        ("near_nnz", C.c_int64),
        ("p2m_rows", C.c_int64),
        ("n_quad_points", C.c_int64),
        ("n_m2l_offsets", C.c_int32),
        ("setup_seconds", C.c_double),
        ("octree_on_device", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PibemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pibem error {code}: {msg}")
        self.code = code


EXPORTS = [
    "pibem_params_default", "pibem_params_from_prm", "pibem_create", "pibem_destroy",
    "pibem_last_error", "pibem_set_stream", "pibem_set_mesh", "pibem_set_bc",
    "pibem_fmm_matvec", "pibem_compute_alpha", "pibem_system_matvec", "pibem_compute_rhs",
    "pibem_solve", "pibem_solve_device", "pibem_tree_info_get", "pibem_tree_boxes",
    "pibem_tree_list", "pibem_tree_list_sublevels", "pibem_near_nnz", "pibem_near_export",
    "pibem_quad_points", "pibem_last_phase_ms", "pibem_set_profiling", "pibem_phase_totals",
    "pibem_launch_count", "pibem_fmm_matvec_noalloc", "pibem_device_bytes",
    "pibem_ucd_read", "pibem_mesh_io_error", "pibem_double_nodes",
    "pibem_dirichlet_mask_from_materials", "pibem_compute_normals",
    "pibem_compute_surface_gradients", "pibem_compute_gradients", "pibem_setup_phases",
    "pibem_slots_open", "pibem_slots_submit", "pibem_slots_step", "pibem_slots_collect",
    "pibem_slots_close", "pibem_apply_preconditioner",
]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)
_lib = None


def load():
    """Load the in-tree CUDA library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    L.pibem_params_default.argtypes = [C.POINTER(Params)]
    L.pibem_params_from_prm.argtypes = [C.POINTER(Params), C.c_char_p]
    L.pibem_create.argtypes = [C.POINTER(Params), C.POINTER(C.c_void_p)]
    L.pibem_destroy.argtypes = [C.c_void_p]
    L.pibem_last_error.restype = C.c_char_p
    L.pibem_last_error.argtypes = [C.c_void_p]
    L.pibem_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.pibem_set_mesh.argtypes = [C.c_void_p, C.c_int64, _dp, C.c_int64, _ip, _ip, _ip]
    L.pibem_set_bc.argtypes = [C.c_void_p, _u8p]
    L.pibem_fmm_matvec.argtypes = [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp]
    L.pibem_compute_alpha.argtypes = [C.c_void_p, _dp]
    L.pibem_system_matvec.argtypes = [C.c_void_p, C.c_int32, _dp, _dp]
    L.pibem_apply_preconditioner.argtypes = [C.c_void_p, C.c_int32, _dp, _dp]
    L.pibem_compute_rhs.argtypes = [C.c_void_p, C.c_int32, _dp, _dp]
    L.pibem_solve.argtypes = [C.c_void_p, C.c_int32, _dp, _dp, _dp, C.POINTER(SolveStats)]
    L.pibem_solve_device.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(SolveStats)]
    L.pibem_tree_info_get.argtypes = [C.c_void_p, C.POINTER(TreeInfo)]
    L.pibem_tree_boxes.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _dp, _ip, _ip]
    L.pibem_tree_list.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _ip, C.c_int32]
    L.pibem_tree_list_sublevels.argtypes = [C.c_void_p, C.c_int32]
    L.pibem_near_nnz.restype = C.c_int64
    L.pibem_near_nnz.argtypes = [C.c_void_p]
    L.pibem_near_export.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp]
    L.pibem_quad_points.argtypes = [C.c_void_p, _dp]
    L.pibem_last_phase_ms.argtypes = [C.c_void_p, _dp]
    L.pibem_set_profiling.argtypes = [C.c_void_p, C.c_int32]
    L.pibem_phase_totals.argtypes = [C.c_void_p, C.c_int32, _dp, C.POINTER(C.c_int64), C.c_int32]
    L.pibem_launch_count.restype = C.c_int64
    L.pibem_launch_count.argtypes = []
    L.pibem_fmm_matvec_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    L.pibem_device_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    L.pibem_ucd_read.argtypes = [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _dp, _ip,
                                 _ip]
    L.pibem_mesh_io_error.restype = C.c_char_p
    L.pibem_mesh_io_error.argtypes = []
    L.pibem_double_nodes.argtypes = [C.c_int64, _dp, C.c_double, _ip, _ip, C.c_int64,
                                     C.POINTER(C.c_int64)]
    L.pibem_dirichlet_mask_from_materials.argtypes = [C.c_int64, C.c_int64, _ip, _ip, C.c_int32,
                                                      _ip, _u8p]
    L.pibem_compute_normals.argtypes = [C.c_void_p, _dp]
    L.pibem_compute_surface_gradients.argtypes = [C.c_void_p, C.c_int32, _dp, _dp]
    L.pibem_compute_gradients.argtypes = [C.c_void_p, C.c_int32, _dp, _dp, _dp]
    L.pibem_setup_phases.argtypes = [C.c_void_p, _dp]
    L.pibem_slots_open.argtypes = [C.c_void_p, C.c_int32]
    L.pibem_slots_submit.argtypes = [C.c_void_p, C.c_int64, _dp, C.POINTER(C.c_int32)]
    L.pibem_slots_step.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.pibem_slots_collect.argtypes = [C.c_void_p, C.POINTER(C.c_int64), _dp, _dp,
                                      C.POINTER(SolveStats)]
    L.pibem_slots_close.argtypes = [C.c_void_p]
    _lib = L
    return L


def launch_count() -> int:
    """Kernels launched by the library so far (all handles)."""
    return int(load().pibem_launch_count())


def default_params(**kw) -> Params:
    p = Params()
    load().pibem_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def params_from_prm(text: str, **kw) -> Params:
    p = default_params()
    rc = load().pibem_params_from_prm(C.byref(p), text.encode())
    if rc:
        raise PibemError(rc, "bad prm text")
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def read_ucd(path: str):
    """UCD (.inp) surface mesh -> (xyz (N,3) float64, cells (C,4) int32 in deal.II
    vertex order, material ids (C,) int32)."""
    L = load()
    nn, nc = C.c_int64(0), C.c_int64(0)
    rc = L.pibem_ucd_read(os.fsencode(path), C.byref(nn), C.byref(nc), None, None, None)
    if rc:
        raise PibemError(rc, L.pibem_mesh_io_error().decode())
    xyz = np.zeros((nn.value, 3))
    cells = np.zeros((nc.value, 4), np.int32)
    mat = np.zeros(nc.value, np.int32)
    rc = L.pibem_ucd_read(os.fsencode(path), C.byref(nn), C.byref(nc), _d(xyz), _i(cells), _i(mat))
    if rc:
        raise PibemError(rc, L.pibem_mesh_io_error().decode())
    return xyz, cells, mat


def double_nodes(xyz, tol: float = 1e-10):
    """Double-node sets of coincident nodes -> (offsets (N+1,), ids) int32 CSR, every
    node's set including itself (the form set_mesh takes)."""
    L = load()
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    n = xyz.shape[0]
    off = np.zeros(n + 1, np.int32)
    tot = C.c_int64(0)
    rc = L.pibem_double_nodes(n, _d(xyz), tol, _i(off), None, 0, C.byref(tot))
    if rc:
        raise PibemError(rc, "double_nodes")
    ids = np.zeros(max(tot.value, 1), np.int32)
    rc = L.pibem_double_nodes(n, _d(xyz), tol, _i(off), _i(ids), len(ids), C.byref(tot))
    if rc:
        raise PibemError(rc, "double_nodes")
    return off, ids[:tot.value]


def dirichlet_mask(n_nodes: int, cells, material, dirichlet_ids):
    """Nodes of cells whose material id is in dirichlet_ids -> 1, others 0."""
    L = load()
    cells = np.ascontiguousarray(cells, np.int32).reshape(-1, 4)
    material = np.ascontiguousarray(material, np.int32)
    ids = np.ascontiguousarray(list(dirichlet_ids) or [0], np.int32)
    mask = np.zeros(n_nodes, np.uint8)
    rc = L.pibem_dirichlet_mask_from_materials(n_nodes, cells.shape[0], _i(cells), _i(material),
                                               len(list(dirichlet_ids)), _i(ids),
                                               mask.ctypes.data_as(_u8p))
    if rc:
        raise PibemError(rc, "dirichlet_mask")
    return mask


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class BEMSolver:
    """One handle: a mesh, its octree and near field, boundary flags, solves."""

    def __init__(self, params: Params | None = None, **kw):
        self.L = load()
        self.params = params if params is not None else default_params(**kw)
        h = C.c_void_p()
        self._check(self.L.pibem_create(C.byref(self.params), C.byref(h)), None)
        self.h = h
        self.n = 0

    def _check(self, rc, h=...):
        if rc != OK:
            hh = self.h if h is ... else h
            msg = self.L.pibem_last_error(hh).decode() if hh else "create failed"
            raise PibemError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            self.L.pibem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None):
        self._check(self.L.pibem_set_stream(self.h, C.c_void_p(stream_ptr or 0)))

    def set_mesh(self, xyz, cells, double_offsets=None, double_ids=None):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
        self.n = self.xyz.shape[0]
        do = None if double_offsets is None else np.ascontiguousarray(double_offsets, np.int32)
        di = None if double_ids is None else np.ascontiguousarray(double_ids, np.int32)
        self._check(self.L.pibem_set_mesh(self.h, self.n, _d(self.xyz), self.cells.shape[0],
                                          _i(self.cells), _i(do) if do is not None else None,
                                          _i(di) if di is not None else None))

    def set_bc(self, dirichlet_mask):
        self.mask = np.ascontiguousarray(dirichlet_mask, dtype=np.uint8)
        self._check(self.L.pibem_set_bc(self.h, self.mask.ctypes.data_as(_u8p)))

    def fmm_matvec(self, phi, dphi_dn):
        phi = np.ascontiguousarray(phi, np.float64)
        dphi = np.ascontiguousarray(dphi_dn, np.float64)
        R = phi.size // self.n
        oN = np.zeros_like(phi)
        oD = np.zeros_like(dphi)
        self._check(self.L.pibem_fmm_matvec(self.h, R, _d(phi), _d(dphi), _d(oN), _d(oD)))
        return oN, oD

    def alpha(self):
        a = np.zeros(self.n)
        self._check(self.L.pibem_compute_alpha(self.h, _d(a)))
        return a

    def system_matvec(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self._check(self.L.pibem_system_matvec(self.h, x.size // self.n, _d(x), _d(y)))
        return y

    def apply_preconditioner(self, v):
        """z = P^-1 v with the handle's preconditioner (PreconditionILU::vmult
        for preconditioner 2)."""
        v = np.ascontiguousarray(v, np.float64)
        z = np.zeros_like(v)
        self._check(self.L.pibem_apply_preconditioner(self.h, v.size // self.n, _d(v), _d(z)))
        return z

    def rhs(self, tmp_rhs):
        t = np.ascontiguousarray(tmp_rhs, np.float64)
        b = np.zeros_like(t)
        self._check(self.L.pibem_compute_rhs(self.h, t.size // self.n, _d(t), _d(b)))
        return b

    def solve(self, tmp_rhs, phi=None, dphi_dn=None, raise_on_noconv=True):
        """BEMProblem::solve_system: returns (phi, dphi_dn, stats)."""
        t = np.ascontiguousarray(tmp_rhs, np.float64)
        R = t.size // self.n
        m = np.tile(self.mask, R).reshape(t.shape)
        phi = np.where(m == 1, t, 0.0) if phi is None else np.array(phi, np.float64)
        dphi = np.where(m == 0, t, 0.0) if dphi_dn is None else np.array(dphi_dn, np.float64)
        st = SolveStats()
        rc = self.L.pibem_solve(self.h, R, _d(phi), _d(dphi), _d(t), C.byref(st))
        if rc == ENOCONV and not raise_on_noconv:
            return phi, dphi, st.as_dict()
        self._check(rc)
        return phi, dphi, st.as_dict()

    # -- request slots (continuous batching, pibem_slots_*) --------------------
    def slots_open(self, max_slots: int):
        self._check(self.L.pibem_slots_open(self.h, int(max_slots)))

    def slots_close(self):
        self._check(self.L.pibem_slots_close(self.h))

    def slots_submit(self, request_id: int, tmp_rhs):
        """Queue one right-hand side (n values); returns its slot, or None when
        every slot is taken."""
        t = np.ascontiguousarray(tmp_rhs, np.float64).reshape(-1)
        slot = C.c_int32(-1)
        rc = self.L.pibem_slots_submit(self.h, int(request_id), _d(t), C.byref(slot))
        if rc == EAGAIN:
            return None
        self._check(rc)
        return int(slot.value)

    def slots_step(self, max_steps: int = 0):
        """Advance the slots; returns (slots in progress, finished slots)."""
        a, d = C.c_int32(0), C.c_int32(0)
        self._check(self.L.pibem_slots_step(self.h, int(max_steps), C.byref(a), C.byref(d)))
        return int(a.value), int(d.value)

    def slots_collect(self):
        """The finished request with the smallest id as (request_id, phi,
        dphi_dn, stats), or None; stats["converged"] is False when it stopped on
        the step limit above the tolerance."""
        rid = C.c_int64(-1)
        phi = np.empty(self.n)
        dphi = np.empty(self.n)
        st = SolveStats()
        rc = self.L.pibem_slots_collect(self.h, C.byref(rid), _d(phi), _d(dphi), C.byref(st))
        if rc == EAGAIN:
            return None
        if rc not in (OK, ENOCONV):
            self._check(rc)
        d = st.as_dict()
        d["converged"] = rc == OK
        return int(rid.value), phi, dphi, d

    def solve_device(self, nrhs, phi_ptr, dphi_ptr, tmp_ptr):
        st = SolveStats()
        self._check(self.L.pibem_solve_device(self.h, nrhs, C.c_void_p(phi_ptr), C.c_void_p(dphi_ptr),
                                              C.c_void_p(tmp_ptr), C.byref(st)))
        return st.as_dict()

    SETUP_PHASES = ("mesh_quadrature", "octree_lists", "plan", "plan_upload", "near_field",
                    "p2m_l2p_tables", "translation_operators", "rest")

    def setup_phases(self):
        """Seconds of each phase of the last set_mesh (dict)."""
        out = np.zeros(len(self.SETUP_PHASES))
        self._check(self.L.pibem_setup_phases(self.h, _d(out)))
        return dict(zip(self.SETUP_PHASES, out.tolist()))

    def tree_info(self):
        ti = TreeInfo()
        self._check(self.L.pibem_tree_info_get(self.h, C.byref(ti)))
        return ti.as_dict()

    def tree(self):
        nb = self.tree_info()["n_boxes"]
        level = np.zeros(nb, np.int32)
        parent = np.zeros(nb, np.int32)
        nchild = np.zeros(nb, np.int32)
        pmin = np.zeros((nb, 3))
        delta = np.zeros(nb)
        nn = np.zeros(nb, np.int32)
        nq = np.zeros(nb, np.int32)
        self._check(self.L.pibem_tree_boxes(self.h, _i(level), _i(parent), _i(nchild), _d(pmin),
                                            _d(delta), _i(nn), _i(nq)))
        return dict(level=level, parent=parent, nchild=nchild, pmin=pmin, delta=delta,
                    n_nodes=nn, n_quads=nq)

    def lists(self, box, kind):
        ns = self.L.pibem_tree_list_sublevels(self.h, box)
        out = []
        buf = np.zeros(4096, np.int32)
        for sub in range(ns):
            k = self.L.pibem_tree_list(self.h, kind, box, sub, _i(buf), len(buf))
            if k > len(buf):
                buf = np.zeros(k, np.int32)
                k = self.L.pibem_tree_list(self.h, kind, box, sub, _i(buf), len(buf))
            out.append(buf[:k].copy())
        return out

    def near(self):
        nnz = self.L.pibem_near_nnz(self.h)
        r = np.zeros(nnz, np.int32)
        c = np.zeros(nnz, np.int32)
        N = np.zeros(nnz)
        D = np.zeros(nnz)
        self._check(self.L.pibem_near_export(self.h, _i(r), _i(c), _d(N), _d(D)))
        return r, c, N, D

    def quad_points(self):
        nq = self.tree_info()["n_quad_points"]
        pts = np.zeros((nq, 3))
        self._check(self.L.pibem_quad_points(self.h, _d(pts)))
        return pts

    PHASES = ["near", "p2m", "m2m", "m2l", "l2l", "m2p", "l2p"]

    def phase_ms(self):
        out = np.zeros(7)
        self._check(self.L.pibem_last_phase_ms(self.h, _d(out)))
        return dict(zip(self.PHASES, out.tolist()))

    # L2 projections onto the Q1 space (BEMProblem::compute_normals /
    # compute_surface_gradients / compute_gradients): (N, 3) arrays, or (R, N, 3)
    def normals(self):
        out = np.zeros((self.n, 3))
        self._check(self.L.pibem_compute_normals(self.h, _d(out)))
        return out

    def surface_gradients(self, u):
        u = np.ascontiguousarray(u, np.float64)
        R = u.size // self.n
        out = np.zeros((R, self.n, 3))
        self._check(self.L.pibem_compute_surface_gradients(self.h, R, _d(u), _d(out)))
        return out[0] if u.ndim == 1 else out

    def gradients(self, phi, dphi_dn):
        phi = np.ascontiguousarray(phi, np.float64)
        dphi = np.ascontiguousarray(dphi_dn, np.float64)
        R = phi.size // self.n
        out = np.zeros((R, self.n, 3))
        self._check(self.L.pibem_compute_gradients(self.h, R, _d(phi), _d(dphi), _d(out)))
        return out[0] if phi.ndim == 1 else out

    def device_bytes(self) -> int:
        """Device memory the handle holds now (bytes)."""
        b = C.c_uint64(0)
        self._check(self.L.pibem_device_bytes(self.h, C.byref(b)))
        return int(b.value)

    def set_profiling(self, on):
        """0 / False off, 1 / True phase timing, 2 phase timing behind a hold
        kernel (GPU execution times without host launch gaps)."""
        self._check(self.L.pibem_set_profiling(self.h, int(on)))

    def phase_totals(self, precision: int, reset: bool = False):
        """(dict phase -> total ms, number of operator applications)."""
        out = np.zeros(7)
        cnt = C.c_int64(0)
        self._check(self.L.pibem_phase_totals(self.h, precision, _d(out), C.byref(cnt), int(reset)))
        return dict(zip(self.PHASES, out.tolist())), int(cnt.value)
