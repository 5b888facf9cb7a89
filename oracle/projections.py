"""Test infrastructure (oracle): CPU restatement of pi-BEM's post-solve L2
projections, used only by tests/ to check the CUDA ones.

    BEMProblem::compute_normals            source/bem_problem.cc:1998-2070
    BEMProblem::compute_surface_gradients  source/bem_problem.cc:1879-1996
    BEMProblem::compute_gradients          source/bem_problem.cc:1747-1877

Each projects a vector field g onto the continuous Q1 space of the mesh, per
component: M u = b with M_ij = sum over cells and Gauss points of
phi_i phi_j JxW and b_i = sum phi_i g JxW.  The FE quantities deal.II's FEValues
gives for FE_Q(1) on the bilinear map of a codimension-one mesh are restated:
shape values, JxW = |x_xi x x_eta| w, the normal x_xi x x_eta / |.|, and
tangential gradients J (J^T J)^-1 grad_ref.  The reference's GMRES + AMG solve is
replaced by a sparse direct solve (the projection is the same).

Parity unpinned against the reference itself (deal.II is absent); pinned by
analytic limits in the tests (sphere normals, gradients of harmonic fields).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def gauss_01(order: int):
    """Tensor Gauss-Legendre rule on [0,1]^2: points (nq, 2), weights (nq,)."""
    x, w = np.polynomial.legendre.leggauss(order)
    x = 0.5 * (x + 1.0)
    w = 0.5 * w
    X, Y = np.meshgrid(x, x, indexing="ij")
    W = np.outer(w, w)
    return np.stack([X.ravel(), Y.ravel()], axis=1), W.ravel()


def _cell_quantities(xyz, cells, order):
    pts, w = gauss_01(order)
    xi, eta = pts[:, 0], pts[:, 1]
    N = np.stack([(1 - xi) * (1 - eta), xi * (1 - eta), (1 - xi) * eta, xi * eta], axis=1)
    dxi = np.stack([-(1 - eta), 1 - eta, -eta, eta], axis=1)
    deta = np.stack([-(1 - xi), -xi, 1 - xi, xi], axis=1)
    v = xyz[cells]                                   # (C, 4, 3)
    tx = np.einsum("qa,cak->cqk", dxi, v)            # (C, nq, 3)
    ty = np.einsum("qa,cak->cqk", deta, v)
    cr = np.cross(tx, ty)
    J = np.linalg.norm(cr, axis=2)
    nrm = cr / J[:, :, None]
    jxw = J * w[None, :]
    g11 = (tx * tx).sum(2)
    g12 = (tx * ty).sum(2)
    g22 = (ty * ty).sum(2)
    det = g11 * g22 - g12 * g12
    # tangential gradients of the shape functions: (C, nq, 4, 3)
    cx = (g22[:, :, None] * dxi[None] - g12[:, :, None] * deta[None]) / det[:, :, None]
    ce = (-g12[:, :, None] * dxi[None] + g11[:, :, None] * deta[None]) / det[:, :, None]
    grad = cx[..., None] * tx[:, :, None, :] + ce[..., None] * ty[:, :, None, :]
    return N, jxw, nrm, grad


def mass_matrix(xyz, cells, order=4):
    N, jxw, _, _ = _cell_quantities(xyz, cells, order)
    Mc = np.einsum("qa,qb,cq->cab", N, N, jxw)
    rows = np.repeat(cells, 4, axis=1).ravel()
    cols = np.tile(cells, (1, 4)).ravel()
    n = len(xyz)
    return sp.coo_matrix((Mc.ravel(), (rows, cols)), shape=(n, n)).tocsc()


def project(xyz, cells, mode, u=None, dudn=None, order=4):
    """mode 'normals' | 'surface_gradients' | 'gradients' -> (N, 3)."""
    xyz = np.asarray(xyz, float)
    cells = np.asarray(cells)
    N, jxw, nrm, grad = _cell_quantities(xyz, cells, order)
    if mode == "normals":
        g = nrm
    else:
        uc = np.asarray(u, float)[cells]                     # (C, 4)
        g = np.einsum("ca,cqak->cqk", uc, grad)
        if mode == "gradients":
            dn = np.einsum("qa,ca->cq", N, np.asarray(dudn, float)[cells])
            g = g + nrm * dn[:, :, None]
    bc = np.einsum("qa,cqk,cq->cak", N, g, jxw)              # (C, 4, 3)
    n = len(xyz)
    b = np.zeros((n, 3))
    np.add.at(b, cells.ravel(), bc.reshape(-1, 3))
    M = mass_matrix(xyz, cells, order)
    lu = spla.splu(M)
    return np.stack([lu.solve(b[:, k]) for k in range(3)], axis=1)
