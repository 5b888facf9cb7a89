"""Double body and double-node constraint lines together on the GPU: a box with
sharp edges open at the symmetry plane z = 0 (its four sides and bottom, double
nodes on every edge), mirrored into a closed box.  The library's FMM solve
(both precision paths) is compared with the oracle's dense double-body solve
(bem_problem.cc:958-1135) under the constraint lines of compute_constraints
(bem_problem.cc:1377-1579): within the p = 8 truncation error (1e-3 relative on
the solution), and both reproduce the symmetric point-source field with the
discretisation error of the mesh."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def _open_box(synthetic, n):
    mesh, _, _, face = synthetic.sharp_cube(n)
    keep = face != 4  # drop the +z face; shift so that the open side lies in z = 0
    cells = mesh.cells[keep]
    used = np.unique(cells)
    remap = -np.ones(mesh.n_nodes, np.int64)
    remap[used] = np.arange(len(used))
    xyz = mesh.xyz[used].copy()
    xyz[:, 2] -= 1.0
    nrm = mesh.normals[used]
    cells = remap[cells].astype(np.int32)
    box = synthetic.Mesh(xyz, cells, nrm)
    groups = {}
    for i, x in enumerate(np.round(xyz * n).astype(np.int64)):
        groups.setdefault(tuple(x), []).append(i)
    sets = [None] * len(xyz)
    for g in groups.values():
        for i in g:
            sets[i] = sorted(g)
    off = np.zeros(len(xyz) + 1, np.int32)
    off[1:] = np.cumsum([len(v) for v in sets])
    ids = np.asarray([d for v in sets for d in v], np.int32)
    return box, face[keep], off, ids


def test_double_body_with_constraint_lines(pibem_mod, oracle_mod, synthetic):
    import constraints
    import projections

    box, face, off, ids = _open_box(synthetic, 6)
    n = box.n_nodes
    rng = np.random.Generator(np.random.PCG64(21))
    S = rng.uniform(-0.4, 0.4, size=(4, 3))
    S[:, 2] = rng.uniform(-1.5, -0.5, 4)
    q = rng.uniform(-1.0, 1.0, 4)
    Sm = S.copy()
    Sm[:, 2] = -Sm[:, 2]
    mask = np.zeros(n, np.uint8)
    mask[np.unique(box.cells[face == 0])] = 1  # +x side Dirichlet
    tmp, ph, dn = synthetic.point_source_data(box, mask, np.vstack([S, Sm]), np.concatenate([q, q]))
    sets = constraints.double_sets(n, off, ids)
    nrm = projections.project(box.xyz, box.cells, "normals")
    sg = projections.project(box.xyz, box.cells, "surface_gradients", u=tmp)
    rows, cols, g = constraints.constraint_lines(sets, mask, tmp, nrm, sg)
    assert len(rows) > 0
    o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
    o.set_mesh(box.xyz, box.cells, off, ids)
    o.set_double_body(1, 0.0)
    o.set_bc(mask)
    o.set_constraints(rows, cols, g)
    ophi, odphi, _, r = o.solve(tmp, tol=1e-10, dense=True, max_steps=3000)
    assert r < 1e-10
    osol = np.where(mask == 1, odphi, ophi)
    exact = np.where(mask == 1, dn, ph)
    sols = {}
    for prec in (pibem_mod.PRECISION_FP64, pibem_mod.PRECISION_MIXED):
        gs = pibem_mod.BEMSolver(precision_mode=prec, is_external_flow=1, double_body=1,
                                 symmetry_plane_z_level=0.0, fma_truncation_order=8,
                                 max_nodes_per_childless_block=20, solver_tolerance=1e-10)
        gs.set_mesh(box.xyz, box.cells, off, ids)
        gs.set_bc(mask)
        phi, dphi, st = gs.solve(tmp)
        assert st["relative_residual"] <= 1e-10, st
        sols[prec] = np.where(mask == 1, dphi, phi)
        gs.close()
    assert rel(sols[pibem_mod.PRECISION_MIXED], sols[pibem_mod.PRECISION_FP64]) < 1e-6
    assert rel(sols[pibem_mod.PRECISION_FP64], osol) < 1e-3
    neu = mask == 0
    assert rel(osol[neu], exact[neu]) < 0.05
    assert rel(sols[pibem_mod.PRECISION_FP64][neu], exact[neu]) < 0.05
