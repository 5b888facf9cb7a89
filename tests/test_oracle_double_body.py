"""The double-body operator on the CPU (no GPU needed).

The reference assembles it densely (BEMProblem::_assemble_system_double_body,
source/bem_problem.cc:958-1135): every collocation row adds, for every cell,
the integral over the cell reflected in z = z0 with the regular Gauss rule.
The oracle restates that (oracle/pibem_oracle.cpp integrate_reflected_cell).
The GPU library evaluates it as an FMM over the closed geometry "mesh + its
reflection" (image node n + k carries the value of node k; only the mesh's
own nodes are collocation rows); oracle.mirror_mesh builds the same geometry.

Checks:
  * dense double body == rows 0..n-1 of the dense operator of the mirrored
    geometry applied to [x, x] (to rounding, 1e-13): the FMM form computes the
    reference's operator;
  * the oracle FMM of the mirrored geometry is within the p = 8 truncation
    error of the dense double body (1e-4);
  * the double-body solve reproduces a field symmetric about the plane (point
    sources inside the wetted Wigley hull and their images) with O(h) error,
    while the one-body operator of the same open surface does not."""
import numpy as np
import pytest

from conftest import rel


@pytest.fixture(scope="module")
def case(synthetic):
    return synthetic.wigley_double_body_case(24, 6)


def test_mirrored_geometry_is_the_reference_operator(oracle_mod, case):
    mesh = case[0]
    n = mesh.n_nodes
    rng = np.random.Generator(np.random.PCG64(11))
    a, b = rng.normal(size=n), rng.normal(size=n)
    o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_double_body(1, 0.0)
    N1, D1 = o.dense_matvec(a, b)
    x2, c2, off, ids = oracle_mod.mirror_mesh(mesh.xyz, mesh.cells, 0.0)
    o2 = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
    o2.set_mesh(x2, c2, off, ids)
    N2, D2 = o2.dense_matvec(np.concatenate([a, a]), np.concatenate([b, b]))
    assert rel(N2[:n], N1) < 1e-13
    assert rel(D2[:n], D1) < 1e-13
    N3, D3 = o2.fmm_matvec(np.concatenate([a, a]), np.concatenate([b, b]))
    assert rel(N3[:n], N1) < 1e-4
    assert rel(D3[:n], D1) < 1e-4
    # the reflected part is not small: the one-body operator differs at O(1)
    o.set_double_body(0)
    N0, D0 = o.dense_matvec(a, b)
    assert rel(N0, N1) > 0.05 and rel(D0, D1) > 0.05


def test_mirror_mesh_layout(oracle_mod, case):
    mesh = case[0]
    n, C = mesh.n_nodes, mesh.n_cells
    x2, c2, off, ids = oracle_mod.mirror_mesh(mesh.xyz, mesh.cells, 0.3)
    assert x2.shape == (2 * n, 3) and c2.shape == (2 * C, 4)
    np.testing.assert_array_equal(x2[n:, :2], mesh.xyz[:, :2])
    np.testing.assert_allclose(x2[n:, 2], 0.6 - mesh.xyz[:, 2], rtol=0, atol=1e-15)
    np.testing.assert_array_equal(c2[C:], mesh.cells[:, [0, 2, 1, 3]] + n)
    assert off[-1] == 2 * n and list(ids[:3]) == [0, 1, 2] and ids[n] == n


@pytest.mark.parametrize("nx,nz", [(24, 6), (48, 12)])
def test_double_body_solve_reproduces_symmetric_field(oracle_mod, synthetic, nx, nz):
    mesh, mask, tmp, ph, dn = synthetic.wigley_double_body_case(nx, nz)
    errs = {}
    for db in (1, 0):
        o = oracle_mod.Oracle(p=8, max_nodes=20, external=True)
        o.set_mesh(mesh.xyz, mesh.cells)
        o.set_double_body(db, 0.0)
        o.set_bc(mask)
        phi, dphi, it, r = o.solve(tmp, tol=1e-10, dense=True)
        assert r < 1e-10
        neu, dr = mask == 0, mask == 1
        errs[db] = (rel(phi[neu], ph[neu]), rel(dphi[dr], dn[dr]))
    bound = 0.06 if nx == 24 else 0.03
    assert errs[1][0] < bound and errs[1][1] < 6 * bound, errs
    assert errs[0][1] > 1.0, errs
