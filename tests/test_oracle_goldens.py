"""Pins the oracle to the reference (CPU).

1. The reference's own golden-output tests (tests/*.output, p = 6): the oracle's
   expansion operators reproduce every printed number.
2. Golden vectors generated by the reference's compiled expansion classes
   (tests/golden/make_golden.py) at p in {4, 6, 8, 10}: the oracle agrees to
   1e-12 relative.
3. Where the reference checkout exists, its compiled classes reproduce the
   .output files line for line.
"""
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
from conftest import reference_dir

REF = reference_dir()


@pytest.fixture(scope="module")
def prims(oracle_mod):
    return oracle_mod.Primitives("oracle")


@pytest.fixture(scope="module")
def outputs():
    with open(os.path.join(GOLD, "reference_test_outputs.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def vectors():
    return dict(np.load(os.path.join(GOLD, "expansion_vectors.npz")))


FIVE = np.array([[2.8, 3.0, 3.0], [3.0, 2.8, 3.0], [3.0, 3.0, 2.8], [3.2, 3.0, 3.0], [3.0, 3.0, 3.2]])
Q5 = np.array([0.1, 0.4, 1.0, 0.2, 0.7])
C = np.array([3.0, 3.0, 3.0])
ZERO = np.zeros(3)


def _six(x):
    """Round to the 6 significant digits the reference log prints."""
    return float(f"{x:.6g}")


def _check(vals, exact, approx):
    assert _six(exact) == pytest.approx(vals["exact"], rel=1e-6)
    assert _six(approx) == pytest.approx(vals["approx"], rel=1e-6)
    assert _six(abs(exact - approx)) == pytest.approx(vals["abs_err"], rel=1e-5)
    assert _six(abs(exact - approx) / abs(exact)) == pytest.approx(vals["rel_err"], rel=1e-5)


def test_multipole_expansion_creation_and_evaluation(prims, outputs):
    exact = float(np.sum(Q5 / np.linalg.norm(FIVE, axis=1)))
    M = prims.p2m(6, C, FIVE, Q5)
    _check(outputs["multipole_expansion_creation_and_evaluation"], exact, prims.m2p(6, C, M, ZERO))


def test_multipole_expansion_translation(prims, outputs):
    exact = float(np.sum(Q5 / np.linalg.norm(FIVE, axis=1)))
    M = prims.p2m(6, C, FIVE, Q5)
    P = prims.m2m(6, C, M, np.array([4.0, 4.0, 4.0]))
    _check(outputs["multipole_expansion_translation"], exact,
           prims.m2p(6, np.array([4.0, 4.0, 4.0]), P, ZERO))


def test_local_expansion_creation_and_translation(prims, outputs):
    exact = float(np.sum(Q5 / np.linalg.norm(FIVE, axis=1)))
    M = prims.p2m(6, C, FIVE, Q5)
    c1, c2 = np.full(3, -2.0), np.full(3, -1.0)
    L = prims.m2l(6, C, M, c1)
    _check(outputs["local_expansion_creation_and_evaluation"], exact, prims.l2p(6, c1, L, ZERO))
    L2 = prims.l2l(6, c1, L, c2)
    _check(outputs["local_expansion_translation"], exact, prims.l2p(6, c2, L2, ZERO))


def test_multipole_expansion_neumann_kernel(prims, outputs):
    pts = np.array([[2.8, 3.0, 3.0], [3.0, 2.8, 3.0], [3.2, 3.0, 2.8], [3.2, 3.0, 3.0], [2.7, 3.0, 3.2]])
    nrm = np.tile([1.0, 0.0, 0.0], (5, 1))
    exact = float(np.sum(-Q5 * (pts * nrm).sum(1) / np.linalg.norm(pts, axis=1) ** 3))
    M = prims.p2m_dipole(6, C, pts, nrm, Q5)
    _check(outputs["multipole_expansion_creation_and_evaluation_neumann_kernel"], exact,
           prims.m2p(6, C, M, ZERO))


def test_copy_goldens(outputs):
    assert outputs["multipole_expansion_copy"]["copy_diff"] == [0.0, 0.0]
    assert outputs["local_expansion_copy"]["copy_diff"] == [0.0, 0.0]


def test_legendre_matches_reference_closed_forms(prims, vectors):
    xs = vectors["leg_x"]
    for n in range(21):
        for m in range(n + 1):
            ref = vectors["leg"][n, m]
            got = np.array([prims.legendre(n, m, x) for x in xs])
            assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
            dref = vectors["dleg"][n, m]
            dgot = np.array([prims.legendre_deriv(n, m, x) for x in xs])
            assert np.abs(dgot - dref).max() <= 1e-11 * max(1.0, np.abs(dref).max())


@pytest.mark.parametrize("p", [4, 6, 8, 10])
@pytest.mark.parametrize("case", [0, 1, 2])
def test_expansion_operators_match_reference(prims, vectors, p, case):
    k = f"p{p}_c{case}_"
    v = {name[len(k):]: val for name, val in vectors.items() if name.startswith(k)}

    def close(a, b, tol=1e-12):
        assert np.abs(a - b).max() <= tol * np.abs(b).max()

    M = prims.p2m(p, v["center"], v["pts"], v["q"])
    close(M, v["p2m"])
    Md = prims.p2m_dipole(p, v["center"], v["pts"], v["normals"], v["q"])
    close(Md, v["p2m_dipole"])
    close(prims.m2m(p, v["center"], v["p2m"], v["parent"]), v["m2m"])
    close(prims.m2l(p, v["center"], v["p2m_dipole"], v["target"]), v["m2l"])
    close(prims.l2l(p, v["target"], v["m2l"], v["child"]), v["l2l"])
    assert prims.m2p(p, v["center"], v["p2m_dipole"], v["x"]) == pytest.approx(float(v["m2p"]), rel=1e-12)
    assert prims.l2p(p, v["target"], v["m2l"], v["x"]) == pytest.approx(float(v["l2p"]), rel=1e-12)


@pytest.mark.skipif(REF is None, reason="reference checkout not present")
def test_compiled_reference_reproduces_output_files():
    repo = os.path.dirname(HERE)
    subprocess.run(["make", "-s", "-C", os.path.join(repo, "oracle"), "ref", f"REF={REF}"], check=True)
    exe = os.path.join(repo, "oracle", "_ref", "ref_goldens")
    with open(os.path.join(GOLD, "reference_test_outputs.json")) as f:
        names = list(json.load(f))
    for sc in names:
        ran = subprocess.run([exe, sc], capture_output=True, text=True, check=True).stdout
        with open(os.path.join(REF, "tests", sc + ".output")) as f:
            assert ran == f.read(), sc
