"""The L2 projections on the GPU (pibem_compute_normals / _surface_gradients /
_gradients) against the CPU restatement (oracle/projections.py) on the same
mesh: 1e-10 relative (2-norm) -- the two differ only in summation order and in
the CG (GPU, to 1e-13) versus direct (CPU) solve.  Meshes include the Wigley
hull, whose collapsed lid cells list a node twice."""
import numpy as np
import pytest

import projections as P
from conftest import rel

pytestmark = pytest.mark.gpu


def _meshes(S):
    return {"sphere": S.cube_sphere(10), "perturbed": S.perturbed_sphere(9, seed=3),
            "wigley": S.wigley_hull(30, 8, 5)}


@pytest.mark.parametrize("name", ["sphere", "perturbed", "wigley"])
def test_projections_match_oracle(name, pibem_mod, synthetic):
    mesh = _meshes(synthetic)[name]
    g = pibem_mod.BEMSolver(fma_truncation_order=4, max_nodes_per_childless_block=30)
    g.set_mesh(mesh.xyz, mesh.cells)
    rng = np.random.Generator(np.random.PCG64(1))
    u = np.stack([np.cos(mesh.xyz @ rng.normal(size=3)) for _ in range(2)])
    dn = rng.normal(size=(2, mesh.n_nodes))
    n_gpu = g.normals()
    n_cpu = P.project(mesh.xyz, mesh.cells, "normals")
    assert rel(n_gpu, n_cpu) < 1e-10
    sg = g.surface_gradients(u)
    gr = g.gradients(u, dn)
    for r in range(2):
        assert rel(sg[r], P.project(mesh.xyz, mesh.cells, "surface_gradients", u[r])) < 1e-10
        assert rel(gr[r], P.project(mesh.xyz, mesh.cells, "gradients", u[r], dn[r])) < 1e-10
    # one column alone gives the same projection, bit for bit (a converged
    # column takes no further CG steps)
    np.testing.assert_array_equal(g.gradients(u[1], dn[1]), gr[1])
    np.testing.assert_array_equal(g.surface_gradients(u[0]), sg[0])
    g.close()
