"""ctypes binding of the oracle (liboracle.so) and of the reference's own
expansion classes (_ref/libpibem_ref.so, present only where the reference
checkout was available at build time).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, only to check or time against it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libpibem_ref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_ucp = C.POINTER(C.c_ubyte)


def build(ref: bool = False) -> None:
    """Compile the oracle (and the reference classes when ref=True)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int] * 6
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_mesh.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, _ip, _ip]
        L.orc_set_bc.argtypes = [C.c_void_p, _ucp]
        L.orc_set_double_body.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.orc_set_constraints.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _dp]
        for f in ("orc_fmm_matvec", "orc_dense_matvec"):
            getattr(L, f).argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_compute_alpha.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_system_matvec.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.orc_compute_rhs.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, _dp]
        L.orc_set_preconditioner.argtypes = [C.c_void_p, C.c_int]
        L.orc_preconditioner_build.restype = C.c_int64
        L.orc_preconditioner_build.argtypes = [C.c_void_p, C.c_int]
        L.orc_preconditioner_apply.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_ilu_factors.argtypes = [C.c_void_p, C.POINTER(C.c_int64), _ip, _dp]
        L.orc_num_blocks.argtypes = [C.c_void_p]
        L.orc_num_levels.argtypes = [C.c_void_p]
        L.orc_level_range.argtypes = [C.c_void_p, _ip, _ip]
        L.orc_block_info.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _dp, _ip, _ip]
        L.orc_childless.argtypes = [C.c_void_p, _ip]
        L.orc_list_sublevels.argtypes = [C.c_void_p, C.c_int]
        L.orc_list.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _ip, C.c_int]
        L.orc_block_nodes.argtypes = [C.c_void_p, C.c_int, _ip, C.c_int]
        L.orc_near_nnz.restype = C.c_long
        L.orc_near_nnz.argtypes = [C.c_void_p]
        L.orc_near_export.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp]
        L.orc_block_expansions.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_num_quad_points.argtypes = [C.c_void_p]
        L.orc_quad_data.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.orc_legendre.restype = C.c_double
        L.orc_legendre.argtypes = [C.c_int, C.c_int, C.c_double]
        L.orc_legendre_deriv.restype = C.c_double
        L.orc_legendre_deriv.argtypes = [C.c_int, C.c_int, C.c_double]
        L.orc_p2m.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, _dp]
        L.orc_p2m_dipole.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, _dp, _dp]
        for f in ("orc_m2m", "orc_m2l", "orc_l2l"):
            getattr(L, f).argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        for f in ("orc_m2p", "orc_l2p"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_gauss_rule.argtypes = [C.c_int, _dp, _dp]
        L.orc_telles_rule.argtypes = [C.c_int, C.c_int, _dp, _dp]
        _lib = L
    return _lib


def mirror_mesh(xyz, cells, z0=0.0, double_offsets=None, double_ids=None):
    """The closed geometry of a double body: the mesh followed by its reflection
    in z = z0 (node n + k is the image of node k; cell C + c the image of cell c
    with vertices (v0, v2, v1, v3), which reverses its orientation so that its
    normal is the reflected normal (n_x, n_y, -n_z) of bem_problem.cc:1048-1052).
    Double-node sets are copied onto the images (no node shares a set with an
    image).  Returns (xyz2, cells2, offsets2, ids2).  Fed to the oracle's FMM
    with the values [x, x], rows 0..n-1 are the FMM form of the double-body
    operator."""
    xyz = np.asarray(xyz, np.float64).reshape(-1, 3)
    cells = np.asarray(cells, np.int32).reshape(-1, 4)
    n = xyz.shape[0]
    im = xyz.copy()
    im[:, 2] = 2.0 * z0 - im[:, 2]
    xyz2 = np.vstack([xyz, im])
    cells2 = np.vstack([cells, cells[:, [0, 2, 1, 3]] + n]).astype(np.int32)
    if double_offsets is None:
        sets = [[i] for i in range(n)]
    else:
        sets = [sorted(set([i] + list(double_ids[double_offsets[i]:double_offsets[i + 1]])))
                for i in range(n)]
    sets2 = sets + [[d + n for d in s_] for s_ in sets]
    off = np.zeros(2 * n + 1, np.int32)
    off[1:] = np.cumsum([len(s_) for s_ in sets2])
    ids = np.asarray([d for s_ in sets2 for d in s_], np.int32)
    return xyz2, cells2, off, ids


def ncoef(p):
    return (p + 1) * (p + 2) // 2


class Oracle:
    """CPU restatement of the reference FMM/dense operators and solve."""

    def __init__(self, p=4, levels=10, max_nodes=30, qorder=4, sorder=5, external=False,
                 threads=None):
        self.L = lib()
        if threads:
            self.L.orc_set_threads(int(threads))
        self.p = p
        self.h = self.L.orc_create(p, levels, max_nodes, qorder, sorder, int(external))

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    def set_mesh(self, xyz, cells, double_offsets=None, double_ids=None):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32)
        self.n = self.xyz.shape[0]
        do = None if double_offsets is None else np.ascontiguousarray(double_offsets, np.int32)
        di = None if double_ids is None else np.ascontiguousarray(double_ids, np.int32)
        self._keep = (do, di)
        self.L.orc_set_mesh(self.h, self.n, _d(self.xyz), self.cells.shape[0], _i(self.cells),
                            _i(do) if do is not None else None, _i(di) if di is not None else None)

    def set_double_body(self, on, z0=0.0):
        """Dense operator of the double body (bem_problem.cc:958-1135)."""
        self.L.orc_set_double_body(self.h, int(on), float(z0))

    def set_constraints(self, rows, cols, g):
        """Constraint lines of solve() (oracle/constraints.py)."""
        self._con = (np.ascontiguousarray(rows, np.int32), np.ascontiguousarray(cols, np.int32),
                     np.ascontiguousarray(g, np.float64))
        r, c, v = self._con
        self.L.orc_set_constraints(self.h, len(r), _i(r), _i(c), _d(v))

    def set_bc(self, mask):
        self.mask = np.ascontiguousarray(mask, dtype=np.uint8)
        self.L.orc_set_bc(self.h, self.mask.ctypes.data_as(_ucp))

    def fmm_matvec(self, phi, dphi):
        phi = np.ascontiguousarray(phi, np.float64)
        dphi = np.ascontiguousarray(dphi, np.float64)
        oN = np.zeros(self.n)
        oD = np.zeros(self.n)
        self.L.orc_fmm_matvec(self.h, _d(phi), _d(dphi), _d(oN), _d(oD))
        return oN, oD

    def dense_matvec(self, phi, dphi):
        phi = np.ascontiguousarray(phi, np.float64)
        dphi = np.ascontiguousarray(dphi, np.float64)
        oN = np.zeros(self.n)
        oD = np.zeros(self.n)
        self.L.orc_dense_matvec(self.h, _d(phi), _d(dphi), _d(oN), _d(oD))
        return oN, oD

    def alpha(self, dense=False):
        a = np.zeros(self.n)
        self.L.orc_compute_alpha(self.h, int(dense), _d(a))
        return a

    def system_matvec(self, alpha, x, dense=False):
        x = np.ascontiguousarray(x, np.float64)
        alpha = np.ascontiguousarray(alpha, np.float64)
        y = np.zeros(self.n)
        self.L.orc_system_matvec(self.h, int(dense), _d(alpha), _d(x), _d(y))
        return y

    def rhs(self, alpha, tmp, dense=False):
        tmp = np.ascontiguousarray(tmp, np.float64)
        alpha = np.ascontiguousarray(alpha, np.float64)
        b = np.zeros(self.n)
        self.L.orc_compute_rhs(self.h, int(dense), _d(alpha), _d(tmp), _d(b))
        return b

    def solve(self, tmp, tol=1e-8, max_steps=1000, restart=100, dense=False, phi=None, dphi=None,
              block_jacobi=False, ilu=False):
        """GMRES(restart) from x0 = rhs to relative true residual tol; with
        block_jacobi, right-preconditioned by the leaf-block Jacobi inverses;
        with ilu, by the ILU(0) of the near-field system matrix
        (BEMFMA::FMA_preconditioner)."""
        self.L.orc_set_preconditioner(self.h, 2 if ilu else int(block_jacobi))
        tmp = np.ascontiguousarray(tmp, np.float64)
        phi = np.where(self.mask == 1, tmp, 0.0) if phi is None else phi.copy()
        dphi = np.where(self.mask == 0, tmp, 0.0) if dphi is None else dphi.copy()
        res = np.zeros(1)
        its = self.L.orc_solve(self.h, int(dense), _d(phi), _d(dphi), _d(tmp), tol, max_steps,
                               restart, _d(res))
        return phi, dphi, its, float(res[0])

    def preconditioner(self, kind):
        """Builds the preconditioner `kind` (0 none, 1 leaf-block Jacobi, 2
        ILU(0) of the near-field system matrix); returns a function v -> P^-1 v
        and, for the ILU, its factors (ptr, col, val) in place in the CSR."""
        nnz = self.L.orc_preconditioner_build(self.h, int(kind))
        factors = None
        if kind == 2:
            ptr = np.zeros(self.n + 1, np.int64)
            col = np.zeros(nnz, np.int32)
            val = np.zeros(nnz)
            self.L.orc_ilu_factors(self.h, ptr.ctypes.data_as(C.POINTER(C.c_int64)), _i(col), _d(val))
            factors = (ptr, col, val)

        def apply(v):
            v = np.ascontiguousarray(v, np.float64)
            z = np.zeros(self.n)
            self.L.orc_preconditioner_apply(self.h, _d(v), _d(z))
            return z

        return apply, factors

    # -- tree export --------------------------------------------------------
    def tree(self):
        nb = self.L.orc_num_blocks(self.h)
        lv = self.L.orc_num_levels(self.h)
        level = np.zeros(nb, np.int32)
        parent = np.zeros(nb, np.int32)
        nchild = np.zeros(nb, np.int32)
        pmin = np.zeros((nb, 3))
        delta = np.zeros(nb)
        nn = np.zeros(nb, np.int32)
        nq = np.zeros(nb, np.int32)
        self.L.orc_block_info(self.h, _i(level), _i(parent), _i(nchild), _d(pmin), _d(delta),
                              _i(nn), _i(nq))
        s = np.zeros(lv + 1, np.int32)
        e = np.zeros(lv + 1, np.int32)
        self.L.orc_level_range(self.h, _i(s), _i(e))
        cl = np.zeros(nb, np.int32)
        ncl = self.L.orc_childless(self.h, _i(cl))
        return dict(level=level, parent=parent, nchild=nchild, pmin=pmin, delta=delta,
                    n_nodes=nn, n_quads=nq, start=s, end=e, childless=cl[:ncl])

    def lists(self, block, kind):
        out = []
        ns = self.L.orc_list_sublevels(self.h, block)
        buf = np.zeros(4096, np.int32)
        for sub in range(ns):
            k = self.L.orc_list(self.h, kind, block, sub, _i(buf), len(buf))
            if k > len(buf):
                buf = np.zeros(k, np.int32)
                k = self.L.orc_list(self.h, kind, block, sub, _i(buf), len(buf))
            out.append(buf[:k].copy())
        return out

    def block_nodes(self, block):
        buf = np.zeros(self.n, np.int32)
        k = self.L.orc_block_nodes(self.h, block, _i(buf), len(buf))
        return buf[:k].copy()

    def near(self):
        nnz = self.L.orc_near_nnz(self.h)
        r = np.zeros(nnz, np.int32)
        c = np.zeros(nnz, np.int32)
        N = np.zeros(nnz)
        D = np.zeros(nnz)
        self.L.orc_near_export(self.h, _i(r), _i(c), _d(N), _d(D))
        return r, c, N, D

    def block_expansions(self, kind):
        nb = self.L.orc_num_blocks(self.h)
        out = np.zeros((nb, ncoef(self.p), 2))
        self.L.orc_block_expansions(self.h, kind, _d(out))
        return out[..., 0] + 1j * out[..., 1]

    def quad_data(self):
        nq = self.L.orc_num_quad_points(self.h)
        pts = np.zeros((nq, 3))
        nrm = np.zeros((nq, 3))
        jxw = np.zeros(nq)
        self.L.orc_quad_data(self.h, _d(pts), _d(nrm), _d(jxw))
        return pts, nrm, jxw


# -- single-expansion primitives (complex, reference storage) ---------------
def _cplx_out(p):
    return np.zeros((ncoef(p), 2))


def _as2(coef):
    c = np.asarray(coef, dtype=np.complex128)
    return np.ascontiguousarray(np.stack([c.real, c.imag], axis=-1))


def _from2(a):
    return a[:, 0] + 1j * a[:, 1]


class Primitives:
    """P2M/M2M/M2L/L2L/M2P/L2P on single expansions through a C library that
    exports the orc_* (oracle) or ref_* (compiled reference) symbols."""

    def __init__(self, which="oracle"):
        if which == "oracle":
            self.L = lib()
            self.pre = "orc_"
        else:
            if not os.path.exists(REFLIB):
                raise FileNotFoundError(REFLIB)
            L = C.CDLL(REFLIB)
            L.ref_legendre.restype = C.c_double
            L.ref_legendre.argtypes = [C.c_uint, C.c_uint, C.c_double]
            L.ref_legendre_deriv.restype = C.c_double
            L.ref_legendre_deriv.argtypes = [C.c_uint, C.c_uint, C.c_double]
            L.ref_p2m.argtypes = [C.c_uint, _dp, C.c_int, _dp, _dp, _dp]
            L.ref_p2m_dipole.argtypes = [C.c_uint, _dp, C.c_int, _dp, _dp, _dp, _dp]
            for f in ("ref_m2m", "ref_m2l", "ref_l2l"):
                getattr(L, f).argtypes = [C.c_uint, _dp, _dp, _dp, _dp]
            for f in ("ref_m2p", "ref_l2p"):
                getattr(L, f).restype = C.c_double
                getattr(L, f).argtypes = [C.c_uint, _dp, _dp, _dp]
            self.L = L
            self.pre = "ref_"

    def _f(self, name):
        return getattr(self.L, self.pre + name)

    def legendre(self, n, m, x):
        return self._f("legendre")(n, m, x)

    def legendre_deriv(self, n, m, x):
        return self._f("legendre_deriv")(n, m, x)

    def p2m(self, p, c, pts, q):
        c = np.ascontiguousarray(c, np.float64)
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        q = np.ascontiguousarray(q, np.float64)
        out = _cplx_out(p)
        self._f("p2m")(p, _d(c), len(q), _d(pts), _d(q), _d(out))
        return _from2(out)

    def p2m_dipole(self, p, c, pts, normals, q):
        c = np.ascontiguousarray(c, np.float64)
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        nr = np.ascontiguousarray(normals, np.float64).reshape(-1, 3)
        q = np.ascontiguousarray(q, np.float64)
        out = _cplx_out(p)
        self._f("p2m_dipole")(p, _d(c), len(q), _d(pts), _d(nr), _d(q), _d(out))
        return _from2(out)

    def _translate(self, name, p, c0, coef, c1):
        c0 = np.ascontiguousarray(c0, np.float64)
        c1 = np.ascontiguousarray(c1, np.float64)
        a = _as2(coef)
        out = _cplx_out(p)
        self._f(name)(p, _d(c0), _d(a), _d(c1), _d(out))
        return _from2(out)

    def m2m(self, p, c_child, coef, c_parent):
        return self._translate("m2m", p, c_child, coef, c_parent)

    def m2l(self, p, c_src, coef, c_tgt):
        return self._translate("m2l", p, c_src, coef, c_tgt)

    def l2l(self, p, c_parent, coef, c_child):
        return self._translate("l2l", p, c_parent, coef, c_child)

    def m2p(self, p, c, coef, x):
        c = np.ascontiguousarray(c, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        return self._f("m2p")(p, _d(c), _d(_as2(coef)), _d(x))

    def l2p(self, p, c, coef, x):
        c = np.ascontiguousarray(c, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        return self._f("l2p")(p, _d(c), _d(_as2(coef)), _d(x))
