"""The oracle's ILU(0) preconditioner: BEMFMA::FMA_preconditioner
(source/bem_fma.cc:3080-3411) factored as Trilinos' PreconditionILU does at its
defaults (level of fill 0, no diagonal shift; source/bem_problem.cc:1302).

The restatement is pinned by the defining property of ILU(0): with L unit
lower and U upper on the sparsity pattern of the matrix, (L U)_ij = A_ij for
every (i, j) of the pattern.  The matrix is formed here independently from the
oracle's near-field export: N on Neumann and -D on Dirichlet columns, alpha on
the diagonal of Neumann rows, and a constrained row its constraint line
{i: 1, c: +1} (bem_fma.cc:3190-3201).  Iteration counts of right-preconditioned
GMRES(100) against the leaf-block Jacobi and no preconditioner follow."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import rel


def _spheroid(S, oracle_mod):
    mesh, mask, tmp, _, _ = S.spheroid_mixed_case(12, seed=2)
    o = oracle_mod.Oracle(p=6, levels=10, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells)
    o.set_bc(mask)
    return o, mesh, mask, tmp, None


def _cube(S, oracle_mod):
    import constraints
    import projections

    mesh, mask, tmp, _, _, off, ids = S.sharp_cube_case(6)
    sets = constraints.double_sets(mesh.n_nodes, off, ids)
    nrm = projections.project(mesh.xyz, mesh.cells, "normals")
    sg = projections.project(mesh.xyz, mesh.cells, "surface_gradients", u=tmp)
    rows, cols, gv = constraints.constraint_lines(sets, mask, tmp, nrm, sg)
    o = oracle_mod.Oracle(p=6, levels=10, max_nodes=20, external=True)
    o.set_mesh(mesh.xyz, mesh.cells, off, ids)
    o.set_bc(mask)
    o.set_constraints(rows, cols, gv)
    return o, mesh, mask, tmp, (rows, cols)


CASES = {"spheroid": _spheroid, "sharp_cube": _cube}


@pytest.fixture(scope="module", params=list(CASES))
def case(request, synthetic, oracle_mod):
    return CASES[request.param](synthetic, oracle_mod)


def _matrix(o, mesh, mask, lines):
    n = mesh.n_nodes
    r, c, N, D = o.near()
    alpha = o.alpha()
    dirm = np.asarray(mask) == 1
    v = np.where(dirm[c], -D, N) + np.where((r == c) & ~dirm[r], alpha[r], 0.0)
    if lines is not None:
        rows, cols = lines
        keep = ~np.isin(r, rows)
        r, c, v = r[keep], c[keep], v[keep]
        lr = [rows, rows[(cols >= 0) & (cols != rows)]]
        lc = [rows, cols[(cols >= 0) & (cols != rows)]]
        r = np.concatenate([r] + lr)
        c = np.concatenate([c] + lc)
        v = np.concatenate([v, np.ones(len(lr[0]) + len(lr[1]))])
    return sp.csr_matrix((v, (r, c)), shape=(n, n))


def test_ilu0_reproduces_the_matrix_on_its_pattern(case):
    o, mesh, mask, _, lines = case
    n = mesh.n_nodes
    apply, (ptr, col, val) = o.preconditioner(2)
    A = _matrix(o, mesh, mask, lines)
    pat = sp.csr_matrix((np.ones(len(col)), col, ptr), shape=(n, n))
    # the pattern is the matrix's (the near field, or the line; entries that
    # are zero, such as D on coplanar elements, stay in it)
    Ab = A.copy()
    Ab.data[:] = 1.0
    assert pat.nnz == A.nnz and abs(pat - Ab).max() == 0
    F = sp.csr_matrix((val, col, ptr), shape=(n, n))
    L = sp.tril(F, -1) + sp.eye(n)
    U = sp.triu(F)
    LU = (L @ U).tocsr()
    assert abs((LU - A).multiply(pat)).max() <= 1e-12 * abs(A).max()
    v = np.random.Generator(np.random.PCG64(3)).normal(size=n)
    assert rel(LU @ apply(v), v) < 1e-12


def test_iteration_counts_against_block_jacobi(case):
    """ILU(0) needs fewer GMRES iterations than the leaf-block Jacobi, which
    needs fewer than none; the three solutions agree."""
    o, mesh, mask, tmp, _ = case
    its, sols = {}, {}
    for name, kw in (("none", {}), ("block_jacobi", dict(block_jacobi=True)), ("ilu", dict(ilu=True))):
        phi, dphi, k, res = o.solve(tmp, tol=1e-10, max_steps=2000, **kw)
        assert res <= 1e-10
        its[name], sols[name] = k, np.where(mask == 1, dphi, phi)
    print("GMRES(100) iterations to 1e-10:", its)
    assert its["ilu"] < its["block_jacobi"] < its["none"]
    assert rel(sols["ilu"], sols["none"]) < 1e-7
    assert rel(sols["block_jacobi"], sols["none"]) < 1e-7
