"""Per-mesh tuning of the octree leaf size and of the FP32 translation engine.

The reference takes `Maximum Number of Collocation Points per Childless Block`
from its parameter file (source/bem_fma.cc:65-103) and has one CPU code path.
Here the best leaf size depends on the order p and on the mesh (near-field
bytes grow with it, far-field translations shrink with it, and the leaf-block
Jacobi preconditioner gets stronger with it), and the FP32 translations can run
on tcgen05 tensor cores or on CUDA cores.  `autotune` times whole solves of a
representative right-hand side for each candidate and returns the fastest
parameters; setup is not timed.  Results are identical in meaning for every
candidate (same operator up to the FMM truncation at the same p, same
tolerance), so the choice only changes speed.
"""
from __future__ import annotations

import time

import numpy as np

import pibem

__all__ = ["autotune"]


def _time_solves(g, tmp, repeats):
    g.solve(tmp)  # warm: allocates the Krylov space, loads the kernels
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        g.solve(tmp)
        best = min(best, time.perf_counter() - t0)
    return best


def autotune(xyz, cells, mask, tmp, leaves=(20, 30, 40, 60),
             engines=(pibem.M2L_TENSOR_CORE, pibem.M2L_CUDA_CORE), repeats=2, **params):
    """Return (best params dict, table of (leaf, engine, seconds per solve)).

    The leaf sizes are timed with the first engine; the other engines are then
    timed at the best leaf size."""
    table = []

    def trial(leaf, engine):
        p = dict(params, max_nodes_per_childless_block=int(leaf), m2l_engine=int(engine))
        g = pibem.BEMSolver(**p)
        try:
            g.set_mesh(xyz, cells)
            g.set_bc(mask)
            t = _time_solves(g, np.asarray(tmp, np.float64), repeats)
        finally:
            g.close()
        table.append((int(leaf), int(engine), t))
        return t

    best_leaf = min(leaves, key=lambda lf: trial(lf, engines[0]))
    best_engine = engines[0]
    t_best = min(t for lf, e, t in table if lf == best_leaf and e == engines[0])
    for e in engines[1:]:
        t = trial(best_leaf, e)
        if t < t_best:
            best_engine, t_best = e, t
    return dict(params, max_nodes_per_childless_block=int(best_leaf),
                m2l_engine=int(best_engine)), table
