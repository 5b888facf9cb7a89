"""Test infrastructure (oracle): CPU restatement of the double-node constraint
lines of pi-BEM's solve, used only by tests/ to check the CUDA library.

    BEMProblem::compute_constraints   source/bem_problem.cc:1377-1579
    ConstrainedOperator (vmult, distribute_rhs)   include/constrained_matrix.h:100-181

For every double-node set (the nodes at one point; each set includes the node)
the "first" node is the first Dirichlet node of the set in ascending id order,
else the smallest id.  Lines are made once per set, when the loop reaches that
first node i:
  * i Neumann: every other node d gets x_d - x_i = 0 (same potential);
  * i Dirichlet, d Neumann: x_d = tmp_rhs[i] (the potential given at i);
  * i Dirichlet, d Dirichlet (normal derivatives on both sides of a sharp edge):
    the reference's flat-edge test divides normal_distance by itself
    (bem_problem.cc:1476), which leaves 1 (or NaN), so the flat branch is never
    taken; with "Continuos gradient across edges" (default true) both lines get
    inhomogeneities from the nodal normals n and the surface gradients s of
    tmp_rhs (L2 projections):  c = n_i . n_d,
        x_i = (s_d . n_i + (s_i . n_d) c) / (1 - c^2)
        x_d = (s_i . n_d + (s_d . n_i) c) / (1 - c^2).
    Adding an existing line is a no-op in deal.II and the inhomogeneity is
    overwritten, so with several Dirichlet doubles x_i keeps the last one's value.
Hanging-node constraints (DoFTools::make_hanging_node_constraints) do not arise
on the conforming meshes the library takes.

constraint_lines returns (rows, cols, g): cols[k] = -1 when the line has no
entry; the only entry weight the reference uses is 1.
"""
from __future__ import annotations

import numpy as np


def double_sets(n, offsets=None, ids=None):
    """Sorted double-node set of every node (the node itself included)."""
    if offsets is None:
        return [[i] for i in range(n)]
    return [sorted(set([i] + [int(v) for v in ids[offsets[i]:offsets[i + 1]]])) for i in range(n)]


def constraint_lines(sets, mask, tmp, normals=None, sgrad=None, continuous_gradient=True):
    lines = {}  # row -> [col, g]
    order = []

    def add_line(row):
        if row not in lines:
            lines[row] = [-1, 0.0]
            order.append(row)

    for i, doubles in enumerate(sets):
        first = doubles[0]
        for d in doubles:
            if mask[d] == 1:
                first = d
                break
        if i != first:
            continue
        others = [d for d in doubles if d != i]
        if mask[i] == 1:
            for d in others:
                if mask[d] == 1:
                    nd = np.float64(np.dot(normals[i], normals[d]))
                    with np.errstate(invalid="ignore", divide="ignore"):
                        nd = nd / nd
                    if nd < 1e-4:  # never true: nd is 1 or NaN
                        add_line(d)
                        lines[d][0] = i
                    elif continuous_gradient:
                        c = float(np.dot(normals[i], normals[d]))
                        s_d_n_i = float(np.dot(sgrad[d], normals[i]))
                        s_i_n_d = float(np.dot(sgrad[i], normals[d]))
                        this = (1.0 / (1.0 - c ** 2)) * (s_d_n_i + s_i_n_d * c)
                        other = (1.0 / (1.0 - c ** 2)) * (s_i_n_d + s_d_n_i * c)
                        add_line(d)
                        add_line(i)
                        lines[i][1] = this
                        add_line(d)
                        lines[d][1] = other
                else:
                    add_line(d)
                    lines[d][1] = float(tmp[i])
        else:
            for d in others:
                add_line(d)
                lines[d][0] = i
    rows = np.asarray(sorted(lines), np.int32)
    cols = np.asarray([lines[r][0] for r in rows], np.int32)
    g = np.asarray([lines[r][1] for r in rows], np.float64)
    return rows, cols, g
