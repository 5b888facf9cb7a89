"""The C++ BEMFMA adapter (include/pibem_bemfma.hpp): compiles against the C ABI
(CPU), and on the GPU drives a solve whose unknowns match the Python binding's."""
import os
import subprocess

import numpy as np
import pytest

from conftest import rel

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "pi-bem_gb300")


def _compile(out):
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "cpp", "adapter_demo.cpp"), "-o", out,
                    "-L", PKG, "-lpibem_gb300", f"-Wl,-rpath,{PKG}"], check=True)


def test_adapter_compiles(tmp_path, pibem_mod):
    pibem_mod.load()  # the library must exist
    _compile(str(tmp_path / "demo"))


@pytest.mark.gpu
def test_adapter_solve_matches_python_binding(tmp_path, pibem_mod, synthetic):
    mesh, mask, tmp, exact = synthetic.sphere_dirichlet_case(10)
    f = tmp_path / "case.txt"
    with open(f, "w") as fh:
        fh.write(f"{mesh.n_nodes}\n" + " ".join(f"{v:.17g}" for v in mesh.xyz.ravel()) + "\n")
        fh.write(f"{mesh.n_cells}\n" + " ".join(str(v) for v in mesh.cells.ravel()) + "\n")
        fh.write(" ".join(str(int(v)) for v in mask) + "\n")
        fh.write(" ".join(f"{v:.17g}" for v in tmp) + "\n")
    exe = str(tmp_path / "demo")
    _compile(exe)
    out = subprocess.run([exe, str(f)], capture_output=True, text=True, check=True).stdout.splitlines()
    vals = np.array([[float(x) for x in line.split()] for line in out[1:]])
    g = pibem_mod.BEMSolver(fma_truncation_order=4, max_nodes_per_childless_block=30)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    phi, dphi, st = g.solve(tmp)
    assert rel(vals[:, 1], dphi) < 1e-12
    assert "residual" in out[0]
