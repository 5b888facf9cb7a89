"""GPU operators against the oracle at the full sizes of the benchmark workloads.

  spheroid98k  the 98,306-node prolate spheroid (semi-axes 3,1,1; 6 x 128 x 128
               Q1 cells), p = 8, <= 40 nodes per childless block, mixed
               Dirichlet / Neumann data from 8 seeded point sources, exterior
               problem -- the headline workload of bench.py;
  wigley55k    a Wigley hull closed by its lid (L = 1, B = 0.1, T = 0.0625;
               sides 2 x 288 x 72 + lid 288 x 48 cells, 55,250 nodes), p = 10,
               <= 40 nodes per childless block, mixed data, exterior problem.

Each operator of the library is compared with the oracle (the CPU restatement
of source/bem_fma.cc multipole_matr_vect_products :2391-3072 and of
source/bem_problem.cc compute_alpha / vmult / compute_rhs :1139-1260) on the
same seeded inputs (measured on GB300: FP64 <= 6e-14, FP64-accurate <= 7e-14,
FP32 <= 1e-7):

  octree boxes and the three lists (built on the device)    identical
  FP64 path: FMM matvec, alpha, vmult, rhs                  1e-12 relative (2-norm)
  FP64-accurate operator (float-float translations, the
    tcgen05 BF16-digit M2L): vmult, rhs                      1e-12 relative
  FP32 operator (tcgen05 3xTF32 M2L): vmult                 1e-6 relative

and the solves: the mixed path's reported residual at 1e-8 is the FP64 one
(1e-3 relative), and its solution at residual 1e-10 is within 1e-7 of the FP64
path's solution driven to 1e-12 (whose operator is the oracle's to 1e-10, so
that is the error against the FP64 oracle's solution up to cond(A) * 1e-10)."""
import os

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def _spheroid98k(S):
    mesh, mask, tmp, _, _ = S.spheroid_mixed_case(128, seed=2)
    return dict(mesh=mesh, mask=mask, tmp=tmp, p=8, leaf=40)


def _wigley55k(S):
    mesh, mask, tmp, _, _ = S.wigley_mixed_case(*S.wigley_for_nodes(55000), seed=3)
    return dict(mesh=mesh, mask=mask, tmp=tmp, p=10, leaf=40)


CASES = {"spheroid98k": _spheroid98k, "wigley55k": _wigley55k}


@pytest.fixture(scope="module", params=list(CASES))
def big(request, synthetic, oracle_mod, pibem_mod):
    c = CASES[request.param](synthetic)
    m = c["mesh"]
    o = oracle_mod.Oracle(p=c["p"], levels=10, max_nodes=c["leaf"], external=True,
                          threads=os.cpu_count())
    o.set_mesh(m.xyz, m.cells)
    o.set_bc(c["mask"])
    rng = np.random.Generator(np.random.PCG64(17))
    x = rng.normal(size=m.n_nodes)
    dphi = rng.normal(size=m.n_nodes)
    alpha = o.alpha()
    c.update(name=request.param, oracle=o, x=x, dphi=dphi, alpha=alpha,
             y_o=o.system_matvec(alpha, x), b_o=o.rhs(alpha, c["tmp"]),
             fmm_o=o.fmm_matvec(x, dphi))
    handles = {}

    def handle(mode, tol=1e-8):
        key = (mode, tol)
        if key not in handles:
            g = pibem_mod.BEMSolver(fma_truncation_order=c["p"], num_octree_levels=10,
                                    max_nodes_per_childless_block=c["leaf"], is_external_flow=1,
                                    precision_mode=mode, solver_tolerance=tol,
                                    solver_max_steps=4000)
            g.set_mesh(m.xyz, m.cells)
            g.set_bc(c["mask"])
            handles[key] = g
        return handles[key]

    c["handle"] = handle
    yield c
    for g in handles.values():
        g.close()


def test_tree_and_lists(big, pibem_mod):
    assert big["handle"](pibem_mod.PRECISION_FP64).tree_info()["octree_on_device"] == 1
    to = big["oracle"].tree()
    tg = big["handle"](pibem_mod.PRECISION_FP64).tree()
    for k in ("level", "parent", "nchild", "n_nodes", "n_quads"):
        assert np.array_equal(to[k], tg[k]), k
    assert np.array_equal(to["pmin"], tg["pmin"]) and np.array_equal(to["delta"], tg["delta"])
    g = big["handle"](pibem_mod.PRECISION_FP64)
    for b in range(len(to["level"])):
        for kind in range(3):
            lo, lg = big["oracle"].lists(b, kind), g.lists(b, kind)
            assert len(lo) == len(lg) and all(np.array_equal(a, bb) for a, bb in zip(lo, lg)), (b, kind)


def test_fp64_operators(big, pibem_mod):
    g = big["handle"](pibem_mod.PRECISION_FP64)
    oN, oD = big["fmm_o"]
    gN, gD = g.fmm_matvec(big["x"], big["dphi"])
    errs = dict(fmmN=rel(gN, oN), fmmD=rel(gD, oD), alpha=rel(g.alpha(), big["alpha"]),
                vmult=rel(g.system_matvec(big["x"]), big["y_o"]), rhs=rel(g.rhs(big["tmp"]), big["b_o"]))
    print(big["name"], "fp64 vs oracle", errs)
    assert max(errs.values()) < 1e-12, errs


def test_fp64_accurate_operator(big, pibem_mod):
    g = big["handle"](pibem_mod.PRECISION_FLOAT_FLOAT)
    errs = dict(vmult=rel(g.system_matvec(big["x"]), big["y_o"]), rhs=rel(g.rhs(big["tmp"]), big["b_o"]))
    print(big["name"], "fp64-accurate vs oracle", errs)
    assert max(errs.values()) < 1e-12, errs


def test_fp32_tensor_core_operator(big, pibem_mod):
    g = big["handle"](pibem_mod.PRECISION_MIXED)
    os.environ["PIBEM_MATVEC_FP32"] = "1"
    try:
        y = g.system_matvec(big["x"])
    finally:
        os.environ.pop("PIBEM_MATVEC_FP32", None)
    e = rel(y, big["y_o"])
    print(big["name"], "fp32 tensor-core vs oracle", e)
    assert e < 1e-6, e


def test_solves(big, pibem_mod):
    """The mixed path's reported residual is an FP64 one: at the working
    tolerance 1e-8 it equals b - A x formed with the oracle-pinned FP64 operator
    to 1e-3 relative.  Driven to 1e-10 its solution is within 1e-7 of the FP64
    path's solution at 1e-12."""
    mask, tmp = big["mask"], big["tmp"]
    g64 = big["handle"](pibem_mod.PRECISION_FP64)
    b = g64.rhs(tmp)
    mix = big["handle"](pibem_mod.PRECISION_MIXED, 1e-8)
    pm, dm, sm = mix.solve(tmp)
    true_res = rel(g64.system_matvec(np.where(mask == 1, dm, pm)), b)
    print(big["name"], "mixed at 1e-8:", sm, "true residual", true_res)
    assert sm["relative_residual"] <= 1e-8 and true_res <= 1.001e-8
    assert abs(true_res - sm["relative_residual"]) <= 1e-3 * true_res
    ref = big["handle"](pibem_mod.PRECISION_FP64, 1e-12)
    pr, dr, st = ref.solve(tmp)
    assert st["relative_residual"] <= 1e-12
    u_ref = np.where(mask == 1, dr, pr)
    tight = big["handle"](pibem_mod.PRECISION_MIXED, 1e-10)
    pt, dt, stt = tight.solve(tmp)
    err = rel(np.where(mask == 1, dt, pt), u_ref)
    print(big["name"], "mixed at 1e-10:", stt, "error against FP64 at 1e-12", err)
    assert stt["relative_residual"] <= 1e-10
    assert err < 1e-7, err
