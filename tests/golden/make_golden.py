"""Generates the golden fixtures of this directory from pi-BEM itself.

Needs the reference checkout (default /root/reference, or $PIBEM_REFERENCE):
  1. builds oracle/_ref (the reference's expansion sources compiled unmodified
     against oracle/refshim/dealii_shim.h);
  2. reference_test_outputs.json -- the numbers of the reference's golden-output
     tests (tests/*.output), read from those files, together with the output of
     the compiled reference running the same scenarios (oracle/ref_goldens.cpp),
     which must match them line for line;
  3. expansion_vectors.npz -- seeded random cases at p in {4,6,8,10} of every
     expansion operator (P2M, normal-dipole P2M, M2M, M2L, L2L, M2P, L2P) and of
     the associated Legendre functions, evaluated by the compiled reference.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

SCENARIOS = [
    "multipole_expansion_creation_and_evaluation",
    "multipole_expansion_translation",
    "local_expansion_creation_and_evaluation",
    "local_expansion_translation",
    "multipole_expansion_creation_and_evaluation_neumann_kernel",
    "multipole_expansion_copy",
    "local_expansion_copy",
]


def parse_output(text):
    vals = {}
    for line in text.splitlines():
        m = re.match(r"DEAL::(Exact potential(?: normal gradient)? at point Q\(0,0,0\)): (\S+)", line)
        if m:
            vals["exact"] = float(m.group(2))
        m = re.match(r"DEAL::Approx potential at point Q\(0,0,0\): (\S+)", line)
        if m:
            vals["approx"] = float(m.group(1))
        m = re.match(r"DEAL::The absolute multipole approximation error is: (\S+)", line)
        if m:
            vals["abs_err"] = float(m.group(1))
        m = re.match(r"DEAL::The relative multipole approximation error is: (\S+)", line)
        if m:
            vals["rel_err"] = float(m.group(1))
        m = re.match(r"DEAL::Total difference .*: \((\S+),(\S+)\)", line)
        if m:
            vals["copy_diff"] = [float(m.group(1)), float(m.group(2))]
    return vals


def main():
    ref = os.environ.get("PIBEM_REFERENCE", "/root/reference")
    if not os.path.isdir(ref):
        sys.exit(f"reference checkout not found at {ref}")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={ref}"], check=True)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_goldens")
    out = {}
    for sc in SCENARIOS:
        golden = open(os.path.join(ref, "tests", sc + ".output")).read()
        ran = subprocess.run([exe, sc], capture_output=True, text=True, check=True).stdout
        if ran != golden:
            sys.exit(f"compiled reference does not reproduce tests/{sc}.output")
        out[sc] = parse_output(golden)
    with open(os.path.join(HERE, "reference_test_outputs.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)

    from oracle import Primitives

    R = Primitives("ref")
    rng = np.random.Generator(np.random.PCG64(2024))
    data = {}
    # Legendre functions and derivatives
    xs = np.linspace(-0.97, 0.97, 23)
    leg = np.zeros((21, 21, len(xs)))
    dleg = np.zeros((21, 21, len(xs)))
    for n in range(21):
        for m in range(n + 1):
            for i, x in enumerate(xs):
                leg[n, m, i] = R.legendre(n, m, x)
                dleg[n, m, i] = R.legendre_deriv(n, m, x)
    data["leg_x"] = xs
    data["leg"] = leg
    data["dleg"] = dleg
    for p in (4, 6, 8, 10):
        for case in range(3):
            key = f"p{p}_c{case}"
            c = rng.uniform(-1, 1, 3)
            pts = c + rng.uniform(-0.5, 0.5, (9, 3))
            q = rng.uniform(-1, 1, 9)
            nr = rng.normal(size=(9, 3))
            M = R.p2m(p, c, pts, q)
            Md = R.p2m_dipole(p, c, pts, nr, q)
            cp = c + rng.choice([-0.5, 0.5], 3)
            M2 = R.m2m(p, c, M, cp)
            ct = c + rng.uniform(2.5, 4.0, 3) * rng.choice([-1, 1], 3)
            Lc = R.m2l(p, c, Md, ct)
            cc = ct + rng.choice([-0.25, 0.25], 3)
            L2 = R.l2l(p, ct, Lc, cc)
            xe = ct + rng.uniform(-0.2, 0.2, 3)
            data[key + "_center"] = c
            data[key + "_pts"] = pts
            data[key + "_q"] = q
            data[key + "_normals"] = nr
            data[key + "_p2m"] = M
            data[key + "_p2m_dipole"] = Md
            data[key + "_parent"] = cp
            data[key + "_m2m"] = M2
            data[key + "_target"] = ct
            data[key + "_m2l"] = Lc
            data[key + "_child"] = cc
            data[key + "_l2l"] = L2
            data[key + "_x"] = xe
            data[key + "_m2p"] = np.array(R.m2p(p, c, Md, xe))
            data[key + "_l2p"] = np.array(R.l2p(p, ct, Lc, xe))
    np.savez_compressed(os.path.join(HERE, "expansion_vectors.npz"), **data)
    print("wrote", os.path.join(HERE, "reference_test_outputs.json"),
          os.path.join(HERE, "expansion_vectors.npz"))


if __name__ == "__main__":
    main()
