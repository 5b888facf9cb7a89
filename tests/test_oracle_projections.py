"""The CPU restatement of the L2 projections (oracle/projections.py) against
analytic limits: on the unit sphere the projected normal tends to x / |x| and
the projected gradient of phi = 1/|x - x0| to its exact gradient (and the
surface gradient to its tangential part) as the mesh is refined."""
import numpy as np

import projections as P


def _errs(S, n):
    mesh = S.cube_sphere(n)
    x = mesh.xyz
    nrm = P.project(x, mesh.cells, "normals")
    e_n = np.abs(nrm - x / np.linalg.norm(x, axis=1, keepdims=True)).max()
    x0 = np.array([2.0, 0.5, 0.3])
    d = x - x0
    r = np.linalg.norm(d, axis=1)
    phi = 1.0 / r
    grad = -d / r[:, None] ** 3
    nn = x / np.linalg.norm(x, axis=1, keepdims=True)
    dn = (grad * nn).sum(axis=1)
    g = P.project(x, mesh.cells, "gradients", phi, dn)
    sg = P.project(x, mesh.cells, "surface_gradients", phi)
    tang = grad - nn * dn[:, None]
    e_g = np.linalg.norm(g - grad) / np.linalg.norm(grad)
    e_s = np.linalg.norm(sg - tang) / np.linalg.norm(tang)
    return e_n, e_g, e_s


def test_projections_converge_to_analytic(synthetic):
    e8 = _errs(synthetic, 8)
    e16 = _errs(synthetic, 16)
    for a, b in zip(e8, e16):
        assert b < 0.6 * a, (e8, e16)
    assert e16[0] < 5e-3 and e16[1] < 5e-2 and e16[2] < 5e-2


def test_mass_matrix_integrates_area(synthetic):
    mesh = synthetic.cube_sphere(12)
    M = P.mass_matrix(mesh.xyz, mesh.cells)
    area = M.sum()
    assert abs(area - 4 * np.pi) < 1e-2 * 4 * np.pi
    assert (M - M.T).count_nonzero() == 0 or abs(M - M.T).max() < 1e-15
