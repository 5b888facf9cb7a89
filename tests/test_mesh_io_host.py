"""Mesh ingestion through the C ABI on the CPU: the UCD (.inp) reader (vertex
order, materials, error reporting), double-node sets of coincident nodes and
Dirichlet masks from material ids.  When the reference checkout is present, its
grids/*.inp files are read as well (skipped otherwise)."""
import os

import numpy as np
import pytest

from conftest import reference_dir

_REF = reference_dir()
REF_GRIDS = os.path.join(_REF, "grids") if _REF else ""


def _write_ucd(path, xyz, cells_lex, material):
    with open(path, "w") as f:
        f.write(f"# written by the test\n{len(xyz)} {len(cells_lex)} 0 0 0\n")
        for i, p in enumerate(xyz):
            f.write(f"{i + 1} {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
        for c, (q, m) in enumerate(zip(cells_lex, material)):
            u = [q[0], q[1], q[3], q[2]]  # lexicographic -> counterclockwise
            f.write(f"{c + 1} {m} quad {' '.join(str(v + 1) for v in u)}\n")


def _outward(xyz, cells):
    v = xyz[cells]
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    return ((v.mean(axis=1) - xyz.mean(axis=0)) * n).sum(axis=1)


def test_ucd_round_trip(tmp_path, pibem_mod, synthetic):
    mesh = synthetic.cube_sphere(3)
    mat = np.where(mesh.xyz[mesh.cells][:, :, 2].mean(axis=1) > 0, 2, 1).astype(np.int32)
    path = str(tmp_path / "s.inp")
    _write_ucd(path, mesh.xyz, mesh.cells, mat)
    xyz, cells, m2 = pibem_mod.read_ucd(path)
    np.testing.assert_array_equal(xyz, mesh.xyz)
    np.testing.assert_array_equal(cells, mesh.cells)
    np.testing.assert_array_equal(m2, mat)
    assert (_outward(xyz, cells) > 0).all()


def test_ucd_errors(tmp_path, pibem_mod):
    with pytest.raises(pibem_mod.PibemError, match="cannot open"):
        pibem_mod.read_ucd(str(tmp_path / "missing.inp"))
    bad = tmp_path / "bad.inp"
    bad.write_text("2 1 0 0 0\n1 0 0 0\n2 1 0 0\n1 1 quad 1 2 3 4\n")
    with pytest.raises(pibem_mod.PibemError, match="unknown node"):
        pibem_mod.read_ucd(str(bad))
    bad.write_text("x y\n")
    with pytest.raises(pibem_mod.PibemError, match="header"):
        pibem_mod.read_ucd(str(bad))


def test_double_nodes_of_split_faces(pibem_mod, synthetic):
    mesh = synthetic.cube_sphere(3)
    # give every cell its own copies of its vertices: coincident nodes = cells per vertex
    xyz = mesh.xyz[mesh.cells.reshape(-1)]
    off, ids = pibem_mod.double_nodes(xyz, 1e-12)
    orig = mesh.cells.reshape(-1)
    for i in range(len(xyz)):
        group = ids[off[i]:off[i + 1]]
        assert i in group
        np.testing.assert_array_equal(np.sort(group), np.flatnonzero(orig == orig[i]))
    off1, ids1 = pibem_mod.double_nodes(mesh.xyz, 1e-12)  # no coincident nodes
    np.testing.assert_array_equal(ids1, np.arange(mesh.n_nodes))


def test_dirichlet_mask_from_materials(pibem_mod, synthetic):
    mesh = synthetic.cube_sphere(4)
    mat = (np.arange(mesh.n_cells) % 3).astype(np.int32)
    mask = pibem_mod.dirichlet_mask(mesh.n_nodes, mesh.cells, mat, [2])
    ref = np.zeros(mesh.n_nodes, np.uint8)
    ref[np.unique(mesh.cells[mat == 2])] = 1
    np.testing.assert_array_equal(mask, ref)
    assert pibem_mod.dirichlet_mask(mesh.n_nodes, mesh.cells, mat, []).sum() == 0


@pytest.mark.skipif(not os.path.isdir(REF_GRIDS), reason="reference checkout not present")
def test_reference_grids(pibem_mod):
    xyz, cells, mat = pibem_mod.read_ucd(os.path.join(REF_GRIDS, "coarse_sphere.inp"))
    assert xyz.shape == (8, 3) and cells.shape == (6, 4) and (mat == 1).all()
    assert (_outward(xyz, cells) > 0).all()
    xyz, cells, mat = pibem_mod.read_ucd(os.path.join(REF_GRIDS, "coarse_sphere_double_nodes.inp"))
    off, ids = pibem_mod.double_nodes(xyz, 1e-7)
    sizes = np.diff(off)
    assert sizes.max() > 1  # the file duplicates the nodes of the cube's edges
    for i in range(len(xyz)):
        g = ids[off[i]:off[i + 1]]
        assert np.abs(xyz[g] - xyz[i]).max() <= 1e-7
    for name in ("sphere.inp", "coarse_cube.inp", "naca0012.inp"):
        x2, c2, m2 = pibem_mod.read_ucd(os.path.join(REF_GRIDS, name))
        assert len(x2) > 0 and c2.min() >= 0 and c2.max() < len(x2)
