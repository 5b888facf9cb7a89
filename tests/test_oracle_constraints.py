"""Double-node constraint lines on the CPU (no GPU needed): the oracle's
restatement of BEMProblem::compute_constraints (oracle/constraints.py,
source/bem_problem.cc:1377-1579) and of ConstrainedOperator
(include/constrained_matrix.h) in the oracle solve.

Mesh: a cube with sharp edges whose faces have their own nodes (double nodes on
the edges, triple nodes at the corners), data from point sources inside, +x and
+z faces Dirichlet (so every kind of set occurs: Neumann-Neumann,
Dirichlet-Neumann, Dirichlet-Dirichlet and mixed corners)."""
import os

import numpy as np
import pytest

from conftest import REPO, rel

REF_GRIDS = os.path.join(os.path.dirname(REPO), "reference", "grids")


@pytest.fixture(scope="module")
def cube(synthetic):
    return synthetic.sharp_cube_case(8)


def _lines(oracle_mod, mesh, mask, tmp, off, ids, continuous=True):
    import constraints
    import projections

    sets = constraints.double_sets(mesh.n_nodes, off, ids)
    nrm = projections.project(mesh.xyz, mesh.cells, "normals")
    sg = projections.project(mesh.xyz, mesh.cells, "surface_gradients", u=tmp)
    return sets, nrm, sg, constraints.constraint_lines(sets, mask, tmp, nrm, sg, continuous)


def test_lines_follow_the_reference_rules(oracle_mod, cube):
    mesh, mask, tmp, ph, dn, off, ids = cube
    sets, nrm, sg, (rows, cols, g) = _lines(oracle_mod, mesh, mask, tmp, off, ids)
    line = {int(r): (int(c), float(v)) for r, c, v in zip(rows, cols, g)}
    kinds = set()
    for s_ in sets:
        if len(s_) < 2:
            continue
        dset = [d for d in s_ if mask[d] == 1]
        first = dset[0] if dset else s_[0]
        for d in s_:
            if d == first:
                if mask[first] == 1 and len(dset) > 1:
                    assert d in line
                continue
            c, v = line[d]
            if mask[first] == 0:
                assert c == first and v == 0.0
                kinds.add("NN")
            elif mask[d] == 0:
                assert c == -1 and v == tmp[first]
                kinds.add("DN")
            else:
                # faces meet at right angles: c = 0, x_d = s_first . n_d
                assert c == -1 and abs(v - np.dot(sg[first], nrm[d])) < 1e-12
                kinds.add("DD")
    assert kinds == {"NN", "DN", "DD"}
    # without continuous gradients the Dirichlet-Dirichlet lines are left out
    r2 = _lines(oracle_mod, mesh, mask, tmp, off, ids, continuous=False)[3][0]
    assert set(r2) < set(rows)


def test_constrained_solve(oracle_mod, cube):
    mesh, mask, tmp, ph, dn, off, ids = cube
    rows, cols, g = _lines(oracle_mod, mesh, mask, tmp, off, ids)[3]
    exact = np.where(mask == 1, dn, ph)
    err = {}
    for con in (True, False):
        o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
        o.set_mesh(mesh.xyz, mesh.cells, off, ids)
        o.set_bc(mask)
        if con:
            o.set_constraints(rows, cols, g)
        phi, dphi, it, r = o.solve(tmp, tol=1e-10, dense=True, max_steps=3000)
        assert r < 1e-10
        sol = np.where(mask == 1, dphi, phi)
        if con:
            ent = cols >= 0
            assert np.abs(sol[rows[ent]] - sol[cols[ent]]).max() < 1e-8 * np.abs(sol).max()
            assert np.abs(sol[rows[~ent]] - g[~ent]).max() < 1e-8 * np.abs(sol).max()
        err[con] = (rel(sol[mask == 0], exact[mask == 0]), rel(sol[mask == 1], exact[mask == 1]))
    assert err[True][0] < 0.01 and err[True][1] < 0.045, err
    assert err[True][1] < 0.8 * err[False][1], err


@pytest.mark.skipif(not os.path.isdir(REF_GRIDS), reason="reference checkout not present")
def test_reference_cube_with_double_nodes(oracle_mod, pibem_mod):
    """grids/coarse_cube_double_nodes.inp: 8 corners, three nodes each."""
    import constraints

    xyz, cells, mat = pibem_mod.read_ucd(os.path.join(REF_GRIDS, "coarse_cube_double_nodes.inp"))
    off, ids = pibem_mod.double_nodes(xyz, 1e-7)
    mask = pibem_mod.dirichlet_mask(len(xyz), cells, mat, [1])
    sets = constraints.double_sets(len(xyz), off, ids)
    assert sorted(len(s_) for s_ in sets) == [3] * 24
    nrm = np.zeros((len(xyz), 3))
    rows, cols, g = constraints.constraint_lines(sets, mask, np.ones(len(xyz)), nrm, nrm, False)
    # one line per non-first node of every set (D-D pairs left out here)
    for s_ in sets:
        dset = [d for d in s_ if mask[d] == 1]
        first = dset[0] if dset else s_[0]
        expect = {d for d in s_ if d != first and not (mask[first] == 1 and mask[d] == 1)}
        assert expect <= set(rows)
