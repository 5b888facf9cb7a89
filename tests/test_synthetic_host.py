"""The synthetic meshes are closed, consistently oriented Q1 surfaces (every
edge shared by two cells and traversed once in each direction), for even and
odd grid counts, and the boundary-data helpers give what they promise.  CPU."""
from collections import Counter

import numpy as np
import pytest


def _directed_edges(cells):
    # deal.II lexicographic vertex order: boundary cycle v0 -> v1 -> v3 -> v2 -> v0
    cyc = cells[:, [0, 1, 3, 2]]
    e = []
    for a, b in zip(cyc.T, np.roll(cyc, -1, axis=1).T):
        e.extend(zip(a.tolist(), b.tolist()))
    return [x for x in e if x[0] != x[1]]  # collapsed edges of degenerate lid cells


def _check_closed_oriented(mesh):
    d = Counter(_directed_edges(mesh.cells))
    assert max(d.values()) == 1, "an edge is traversed twice in the same direction"
    for (a, b) in d:
        assert (b, a) in d, f"edge {a}-{b} is on the boundary"
    used = np.zeros(mesh.n_nodes, bool)
    used[mesh.cells.ravel()] = True
    assert used.all()


@pytest.mark.parametrize("dims", [(24, 6, 4), (24, 6, 5), (66, 16, 11), (30, 7, 3)])
def test_wigley_closed_and_oriented(synthetic, dims):
    _check_closed_oriented(synthetic.wigley_hull(*dims))


@pytest.mark.parametrize("n", [3, 8])
def test_spheres_closed_and_oriented(synthetic, n):
    _check_closed_oriented(synthetic.cube_sphere(n))
    _check_closed_oriented(synthetic.perturbed_sphere(n, seed=1))


def test_outward_normals(synthetic):
    S = synthetic
    for mesh in (S.cube_sphere(6), S.perturbed_sphere(6, seed=3), S.wigley_hull(24, 6, 5)):
        c = mesh.xyz.mean(axis=0)
        # mean of (x - c) . n over the nodes is positive for outward normals
        assert ((mesh.xyz - c) * mesh.normals).sum(axis=1).mean() > 0


def test_node_count_helpers(synthetic):
    S = synthetic
    for n in (2000, 20000):
        assert abs(S.wigley_hull(*S.wigley_for_nodes(n)).n_nodes - n) < 0.1 * n
    nx, nz, ny = S.wigley_for_nodes(393000)
    assert (nx, nz, ny) == (768, 192, 128)
    for n in (2000, 20000, 200000):
        k = S.sphere_n_for_nodes(n)
        assert abs(6 * k * k + 2 - n) < 0.1 * n


def test_plane_mask_and_sources(synthetic):
    S = synthetic
    m = S.wigley_hull(30, 8, 6)
    for seed in range(5):
        mask = S.random_plane_mask(m, seed)
        assert 0 < mask.sum() < m.n_nodes
    rng = np.random.Generator(np.random.PCG64(0))
    src = S.sources_in_wigley(rng, 200)
    hb = 0.05 * (1 - (2 * src[:, 0]) ** 2) * (1 - (src[:, 2] / 0.0625) ** 2)
    assert (np.abs(src[:, 1]) < hb).all() and (src[:, 2] < 0).all() and (src[:, 2] > -0.0625).all()
    src = S.sources_in_ball(rng, 200, 0.5)
    assert (np.linalg.norm(src, axis=1) < 0.5).all()


def test_sharp_cube_double_nodes(synthetic):
    """Faces with their own nodes: every double-node set holds nodes at one point;
    edge nodes come in pairs, corners in threes; cells face outward."""
    mesh, off, ids, face = synthetic.sharp_cube(5)
    sizes = np.diff(off)
    assert set(sizes.tolist()) == {1, 2, 3}
    assert (sizes == 3).sum() == 8 * 3
    for i in range(mesh.n_nodes):
        g = ids[off[i]:off[i + 1]]
        assert i in g and np.abs(mesh.xyz[g] - mesh.xyz[i]).max() < 1e-12
    v = mesh.xyz[mesh.cells]
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    assert ((nrm * v.mean(axis=1)).sum(axis=1) > 0).all()
    assert np.bincount(face).tolist() == [25] * 6


def test_wetted_wigley_is_open_at_the_waterline(synthetic):
    """lid=False keeps the two sides only; the waterline nodes lie in z = 0 and
    the double-body case's normals there are horizontal."""
    closed = synthetic.wigley_hull(12, 3, 2)
    wet = synthetic.wigley_hull(12, 3, 2, lid=False)
    assert wet.n_cells == 2 * 12 * 3 and closed.n_cells == wet.n_cells + 12 * 2
    case = synthetic.wigley_double_body_case(12, 3)
    mesh = case[0]
    top = np.abs(mesh.xyz[:, 2]) < 1e-12
    assert top.sum() > 0 and np.abs(mesh.normals[top, 2]).max() < 1e-12
