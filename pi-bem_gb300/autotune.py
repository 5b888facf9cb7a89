"""Per-mesh tuning of the FMM order, the octree leaf size and the tiles of the
FP32 translations.

The reference takes `FMA Truncation Order` and `Maximum Number of Collocation
Points per Childless Block` from its parameter file (source/bem_fma.cc:65-103)
and has one CPU code path.  Here:

* the order p is chosen under an accuracy target: the relative difference of
  the FP64 operator at order p and at the highest candidate order, applied to
  a seeded random vector, must not exceed `accuracy` (the FMM truncation error
  of order p is well estimated by that difference, the higher order's own
  being far smaller); among the orders that meet it, the fastest solve wins;
* the leaf size changes the split between near-field bytes and far-field
  translations and the strength of the leaf-block Jacobi preconditioner;
* the FP32 translations run on tcgen05 tensor cores or on CUDA cores, and the
  tensor-core M2L has two tile knobs: the most pairs of one operator in a tile
  chunk (`m2l_chunk_pairs`) and the depth of its pipeline (`m2l_stages`).

`autotune` times whole solves of a representative right-hand side for each
candidate and returns the fastest parameters; set-up is not timed.  The leaf
size and the tile knobs change speed only (every candidate solves the same
problem at the same order to the same tolerance); the order also changes the
operator, within the accuracy target.
"""
from __future__ import annotations

import time

import numpy as np

import pibem

__all__ = ["autotune", "truncation_error"]


def _handle(xyz, cells, mask, params):
    g = pibem.BEMSolver(**params)
    g.set_mesh(xyz, cells)
    g.set_bc(mask)
    return g


def _time_solves(g, tmp, repeats):
    g.solve(tmp)  # warm: allocates the Krylov space, captures the graphs
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        g.solve(tmp)
        best = min(best, time.perf_counter() - t0)
    return best


def truncation_error(xyz, cells, mask, orders, seed=0, **params):
    """{p: ||A_p x - A_pmax x|| / ||A_pmax x||} for the FP64 system operator
    and a seeded random x (pmax = max(orders))."""
    base = dict(params, precision_mode=pibem.PRECISION_FP64)
    x = np.random.Generator(np.random.PCG64(seed)).normal(size=np.asarray(xyz).reshape(-1, 3).shape[0])
    ys = {}
    for p in sorted(set(orders)):
        g = _handle(xyz, cells, mask, dict(base, fma_truncation_order=int(p)))
        try:
            ys[p] = g.system_matvec(x)
        finally:
            g.close()
    ref = ys[max(ys)]
    return {p: float(np.linalg.norm(y - ref) / np.linalg.norm(ref)) for p, y in ys.items()}


def autotune(xyz, cells, mask, tmp, orders=None, accuracy=1e-5, leaves=(20, 30, 40, 60),
             engines=(pibem.M2L_TENSOR_CORE, pibem.M2L_CUDA_CORE), chunks=(64, 128),
             stages=(2, 3), repeats=2, **params):
    """Return (best params dict, table of trials).

    orders: candidate FMM orders (None: keep params' fma_truncation_order).
    The order is chosen first (the fastest order meeting `accuracy`, timed at
    the first leaf size), then the leaf size, then the engine, then the
    tensor-core tile knobs.  Each trial is (order, leaf, engine, chunk pairs,
    stages, seconds per solve); the table also records the truncation error of
    each order under "errors"."""
    table = []
    tmp = np.asarray(tmp, np.float64)

    def trial(p, leaf, engine, chunk, st):
        prm = dict(params, fma_truncation_order=int(p), max_nodes_per_childless_block=int(leaf),
                   m2l_engine=int(engine), m2l_chunk_pairs=int(chunk), m2l_stages=int(st))
        g = _handle(xyz, cells, mask, prm)
        try:
            t = _time_solves(g, tmp, repeats)
        finally:
            g.close()
        table.append((int(p), int(leaf), int(engine), int(chunk), int(st), t))
        return t

    timed = {}

    def cached(p, leaf, engine, chunk, st):
        k = (p, leaf, engine, chunk, st)
        if k not in timed:
            timed[k] = trial(*k)
        return timed[k]

    errors = {}
    p0 = params.get("fma_truncation_order", 6)
    if orders:
        rest = {k: v for k, v in params.items()
                if k not in ("fma_truncation_order", "max_nodes_per_childless_block")}
        errors = truncation_error(xyz, cells, mask, orders, max_nodes_per_childless_block=leaves[0],
                                  **rest)
        ok = [p for p in sorted(errors) if errors[p] <= accuracy] or [max(errors)]
        p0 = min(ok, key=lambda p: cached(p, leaves[0], engines[0], 0, 0))
    best_leaf = min(leaves, key=lambda lf: cached(p0, lf, engines[0], 0, 0))
    best = dict(engine=engines[0], chunk=0, stages=0)
    t_best = cached(p0, best_leaf, engines[0], 0, 0)
    for e in engines[1:]:
        t = trial(p0, best_leaf, e, 0, 0)
        if t < t_best:
            best, t_best = dict(engine=e, chunk=0, stages=0), t
    if best["engine"] == pibem.M2L_TENSOR_CORE:
        for c in chunks:
            for s in stages:
                t = trial(p0, best_leaf, pibem.M2L_TENSOR_CORE, c, s)
                if t < t_best:
                    best, t_best = dict(engine=pibem.M2L_TENSOR_CORE, chunk=c, stages=s), t
    out = dict(params, fma_truncation_order=int(p0), max_nodes_per_childless_block=int(best_leaf),
               m2l_engine=int(best["engine"]), m2l_chunk_pairs=int(best["chunk"]),
               m2l_stages=int(best["stages"]))
    return out, {"trials": table, "errors": errors}
