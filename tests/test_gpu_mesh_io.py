"""A mesh read from a UCD (.inp) file, with its Dirichlet mask from material ids,
goes through the C ABI exactly like the same mesh given as arrays: identical
solution, bit for bit."""
import numpy as np
import pytest

from test_mesh_io_host import _write_ucd

pytestmark = pytest.mark.gpu


def test_ucd_mesh_solves_like_arrays(tmp_path, pibem_mod, synthetic):
    S = synthetic
    mesh = S.perturbed_sphere(10, seed=7)
    mat = np.where(mesh.xyz[mesh.cells][:, :, 2].mean(axis=1) > 0, 3, 1).astype(np.int32)
    path = str(tmp_path / "m.inp")
    _write_ucd(path, mesh.xyz, mesh.cells, mat)
    xyz, cells, m2 = pibem_mod.read_ucd(path)
    mask = pibem_mod.dirichlet_mask(len(xyz), cells, m2, [3])
    np.testing.assert_array_equal(mask, S.mixed_bc_by_cell_centroid(mesh))
    tmp = S.spheroid_mixed_case(0, seed=5, mesh=mesh)[2]
    sols = []
    for x, c in ((xyz, cells), (mesh.xyz, mesh.cells)):
        g = pibem_mod.BEMSolver(fma_truncation_order=6, max_nodes_per_childless_block=20,
                                is_external_flow=1, precision_mode=pibem_mod.PRECISION_MIXED)
        g.set_mesh(x, c)
        g.set_bc(mask)
        phi, dphi, st = g.solve(tmp)
        assert st["relative_residual"] <= 1e-8
        sols.append((phi, dphi))
        g.close()
    np.testing.assert_array_equal(sols[0][0], sols[1][0])
    np.testing.assert_array_equal(sols[0][1], sols[1][1])
