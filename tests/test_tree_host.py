"""The product's host octree / list builder (pi-bem_gb300/csrc/tree.cpp) against
the oracle's std::set restatement of BEMFMA::generate_octree_blocking
(source/bem_fma.cc:3615-4801), on the CPU: identical box tables (ids, levels,
parents, geometry bit for bit, node and quadrature counts), identical
childless list and identical nearNeigh / intList / nonIntList sets for every
box and sublevel."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARN = os.path.join(REPO, "tests", "harness")


@pytest.fixture(scope="module")
def th(tmp_path_factory):
    out = tmp_path_factory.mktemp("th") / "libth.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
                    "-I/usr/local/cuda/include", "-o", str(out),
                    os.path.join(HARN, "tree_harness.cpp"),
                    os.path.join(REPO, "pi-bem_gb300", "csrc", "tree.cpp")], check=True)
    return C.CDLL(str(out))


dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


def _compare(th, oracle_mod, mesh, p=4, levels=10, leaf=30):
    o = oracle_mod.Oracle(p=p, levels=levels, max_nodes=leaf)
    o.set_mesh(mesh.xyz, mesh.cells)
    pts, _, _ = o.quad_data()
    pts = np.ascontiguousarray(pts)
    nb = th.th_build(mesh.n_nodes, mesh.xyz.ctypes.data_as(dp), mesh.n_cells,
                     mesh.cells.ctypes.data_as(ip), pts.ctypes.data_as(dp), 16, levels, leaf)
    tr = o.tree()
    assert nb == len(tr["level"])
    arr = {k: np.zeros(nb, np.int32) for k in ("level", "parent", "nchild", "n_nodes", "n_quads")}
    pm, de = np.zeros((nb, 3)), np.zeros(nb)
    th.th_boxes(*(arr[k].ctypes.data_as(ip) for k in ("level", "parent", "nchild")),
                pm.ctypes.data_as(dp), de.ctypes.data_as(dp), arr["n_nodes"].ctypes.data_as(ip),
                arr["n_quads"].ctypes.data_as(ip))
    for k, a in arr.items():
        assert np.array_equal(a, tr[k]), k
    assert np.array_equal(pm, tr["pmin"]) and np.array_equal(de, tr["delta"])
    cl = np.zeros(nb, np.int32)
    ncl = th.th_childless(cl.ctypes.data_as(ip))
    assert np.array_equal(cl[:ncl], tr["childless"])
    buf = np.zeros(200000, np.int32)
    for b in range(nb):
        for kind in range(3):
            ol = o.lists(b, kind)
            assert th.th_nsub(b) == len(ol)
            for sub, ref in enumerate(ol):
                k = th.th_list(kind, b, sub, buf.ctypes.data_as(ip), len(buf))
                assert k == len(ref) and np.array_equal(buf[:k], ref), (b, kind, sub)
    return nb


def test_sphere_config1(th, oracle_mod, synthetic):
    mesh = synthetic.cube_sphere(16)
    assert _compare(th, oracle_mod, mesh, leaf=30) > 100


def test_small_leaves_deep_tree(th, oracle_mod, synthetic):
    assert _compare(th, oracle_mod, synthetic.cube_sphere(12), leaf=6, levels=10) > 300


def test_spheroid(th, oracle_mod, synthetic):
    _compare(th, oracle_mod, synthetic.spheroid(20), leaf=20)


def test_perturbed_sphere_shallow_tree(th, oracle_mod, synthetic):
    _compare(th, oracle_mod, synthetic.perturbed_sphere(14, seed=5), leaf=10, levels=5)


def test_wigley_hull(th, oracle_mod, synthetic):
    _compare(th, oracle_mod, synthetic.wigley_hull(40, 8, 6), leaf=20)


def test_double_body_tree_and_plan(th, oracle_mod, synthetic):
    """Double body: the octree of the mirrored geometry equals the oracle's
    for that geometry, and the plan's rows, columns and targets are the mesh's
    own nodes only (image nodes are sources whose values are their
    originals')."""
    mesh = synthetic.wigley_double_body_case(40, 8)[0]
    n = mesh.n_nodes
    x2, c2, _, _ = oracle_mod.mirror_mesh(mesh.xyz, mesh.cells, 0.0)
    geo = synthetic.Mesh(x2, c2, np.zeros_like(x2))
    _compare(th, oracle_mod, geo, leaf=20)
    o = oracle_mod.Oracle(p=4, levels=10, max_nodes=20)
    o.set_mesh(x2, c2)
    pts = np.ascontiguousarray(o.quad_data()[0])
    st = np.zeros(11, np.int64)
    th.th_plan_mirrored.argtypes = [C.c_int, dp, C.c_int, ip, C.c_double, dp, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.POINTER(C.c_long)]
    cells = np.ascontiguousarray(mesh.cells, np.int32)
    th.th_plan_mirrored(n, mesh.xyz.ctypes.data_as(dp), mesh.n_cells, cells.ctypes.data_as(ip), 0.0,
                        pts.ctypes.data_as(dp), 16, 10, 20, 4, st.ctypes.data_as(C.POINTER(C.c_long)))
    assert st[0] == n and st[9] == 0          # every collocation node is one near row
    assert st[1] < n and st[2] < n and st[3] < n
    assert st[4] == n
    assert st[5] > 0 and st[6] == 0 and st[8] == 0 and st[10] == 0
