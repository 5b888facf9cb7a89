"""Synthetic surface meshes and boundary data for the FMM-BEM solve.

The meshes are quadrilateral Q1 surface meshes with shared vertices (no double
nodes), cells given as 4 node ids in deal.II lexicographic vertex order
(v0=(0,0), v1=(1,0), v2=(0,1), v3=(1,1) of the unit cell), oriented so that the
cell normal d x/d xi x d x/d eta points out of the body -- the convention the
reference's collocation operator assumes (source/bem_problem.cc:478-950).

Workloads:
  * unit cube-sphere, 6 x n x n cells (6 n^2 + 2 nodes), Dirichlet data from a
    point source outside the sphere (interior problem);
  * the same cube-sphere scaled to a prolate spheroid (3,1,1), mixed
    Dirichlet (cells with centroid z > 0) / Neumann (z <= 0) data from seeded
    point sources inside the body (exterior problem);
  * a Wigley-type hull closed by a lid, mixed data from point sources inside;
  * perturbed spheres r = 1 + 0.1 * sum_{l<=4} c_lm Y_lm.
All seeds use numpy.random.Generator(PCG64(seed)).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "Mesh",
    "cube_sphere",
    "spheroid",
    "perturbed_sphere",
    "wigley_hull",
    "point_source_field",
    "mixed_bc_by_cell_centroid",
    "sphere_dirichlet_case",
    "spheroid_mixed_case",
    "random_plane_mask",
    "sources_in_ball",
    "sources_in_wigley",
    "point_source_data",
    "wigley_mixed_case",
    "wigley_for_nodes",
    "sphere_n_for_nodes",
]


class Mesh:
    """Nodes (N,3) float64, cells (C,4) int32, analytic outward normals (N,3)."""

    def __init__(self, xyz, cells, normals):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32)
        self.normals = np.ascontiguousarray(normals, dtype=np.float64)

    @property
    def n_nodes(self):
        return self.xyz.shape[0]

    @property
    def n_cells(self):
        return self.cells.shape[0]


def _cube_surface(n: int):
    """Equiangular cube-sphere connectivity on the unit cube surface.

    Returns unit-sphere node positions and cells; vertices on cube edges are
    shared between faces (6 n^2 + 2 nodes)."""
    ticks = np.tan(np.pi / 4 * np.linspace(-1.0, 1.0, n + 1))
    index = {}
    pts = []

    def node(ijk):
        key = tuple(int(v) for v in ijk)
        k = index.get(key)
        if k is None:
            k = len(pts)
            index[key] = k
            pts.append([ticks[key[0]], ticks[key[1]], ticks[key[2]]])
        return k

    cells = []
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        for sign in (1, -1):
            s_ax, t_ax = (b, c) if sign > 0 else (c, b)
            fixed = n if sign > 0 else 0
            for j in range(n):
                for i in range(n):
                    quad = []
                    for dj in (0, 1):
                        for di in (0, 1):
                            ijk = [0, 0, 0]
                            ijk[a] = fixed
                            ijk[s_ax] = i + di
                            ijk[t_ax] = j + dj
                            quad.append(node(ijk))
                    cells.append(quad)
    p = np.asarray(pts, dtype=np.float64)
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    return p, np.asarray(cells, dtype=np.int32)


def sharp_cube(n: int, half: float = 1.0):
    """Cube [-half, half]^3 with sharp edges: every face is its own uniform n x n
    grid with its own nodes, so nodes on the edges and corners are double
    (triple) nodes, as CAD meshes with sharp edges give them.  Outward cells
    (the cube-sphere's orientation).

    Returns (mesh with face normals as nodal normals, double-node CSR offsets,
    ids (every node's set includes itself), face id of every cell: 0..5 for
    +x, -x, +y, -y, +z, -z)."""
    ticks = np.linspace(-half, half, n + 1)
    pts, nrm, cells, face = [], [], [], []
    index = {}
    f = 0
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        for sign in (1, -1):
            s_ax, t_ax = (b, c) if sign > 0 else (c, b)
            fixed = n if sign > 0 else 0
            normal = [0.0, 0.0, 0.0]
            normal[a] = float(sign)
            for j in range(n):
                for i in range(n):
                    quad = []
                    for dj in (0, 1):
                        for di in (0, 1):
                            ijk = [0, 0, 0]
                            ijk[a] = fixed
                            ijk[s_ax] = i + di
                            ijk[t_ax] = j + dj
                            key = (f, *ijk)
                            k = index.get(key)
                            if k is None:
                                k = len(pts)
                                index[key] = k
                                pts.append([ticks[ijk[0]], ticks[ijk[1]], ticks[ijk[2]]])
                                nrm.append(normal)
                            quad.append(k)
                    cells.append(quad)
                    face.append(f)
            f += 1
    xyz = np.asarray(pts, dtype=np.float64)
    groups = {}
    for i, x in enumerate(np.round(xyz / half * n).astype(np.int64)):
        groups.setdefault(tuple(x), []).append(i)
    sets = [None] * len(xyz)
    for g in groups.values():
        for i in g:
            sets[i] = sorted(g)
    off = np.zeros(len(xyz) + 1, np.int32)
    off[1:] = np.cumsum([len(v) for v in sets])
    ids = np.asarray([d for v in sets for d in v], np.int32)
    return (Mesh(xyz, np.asarray(cells, np.int32), np.asarray(nrm)), off, ids,
            np.asarray(face, np.int32))


def sharp_cube_case(n: int, seed: int = 7, n_sources: int = 6, dirichlet_faces=(0, 4)):
    """Sharp cube (double nodes on every edge) with mixed data from n_sources
    point sources of strength U(-1,1) in |s| < 0.5 (exterior problem): the nodes
    of the faces in dirichlet_faces (default +x and +z, which share an edge)
    are Dirichlet, the rest Neumann.

    Returns mesh, dirichlet mask, tmp_rhs, exact phi, exact dphi/dn, double
    offsets, double ids."""
    mesh, off, ids, face = sharp_cube(n)
    rng = np.random.Generator(np.random.PCG64(seed))
    q = rng.uniform(-1.0, 1.0, n_sources)
    S = sources_in_ball(rng, n_sources)
    mask = np.zeros(mesh.n_nodes, np.uint8)
    mask[np.unique(mesh.cells[np.isin(face, dirichlet_faces)])] = 1
    tmp, ph, dn = point_source_data(mesh, mask, S, q)
    return mesh, mask, tmp, ph, dn, off, ids


def cube_sphere(n: int, radius: float = 1.0) -> Mesh:
    p, cells = _cube_surface(n)
    return Mesh(radius * p, cells, p.copy())


def spheroid(n: int, axes=(3.0, 1.0, 1.0)) -> Mesh:
    p, cells = _cube_surface(n)
    ax = np.asarray(axes, dtype=np.float64)
    xyz = p * ax
    nrm = xyz / ax**2
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return Mesh(xyz, cells, nrm)


def _real_sph_harm(l, m, theta, phi):
    """Real spherical harmonics (unnormalised beyond the Legendre factor)."""
    from scipy.special import lpmv

    x = np.cos(theta)
    P = lpmv(abs(m), l, x)
    if m > 0:
        return P * np.cos(m * phi)
    if m < 0:
        return P * np.sin(-m * phi)
    return P


def perturbed_sphere(n: int, seed: int, amp: float = 0.1, lmax: int = 4) -> Mesh:
    p, cells = _cube_surface(n)
    rng = np.random.Generator(np.random.PCG64(seed))
    theta = np.arccos(np.clip(p[:, 2], -1, 1))
    phi = np.arctan2(p[:, 1], p[:, 0])
    s = np.zeros(len(p))
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            s += rng.normal() * _real_sph_harm(l, m, theta, phi)
    s /= max(np.abs(s).max(), 1e-300)
    r = 1.0 + amp * s
    xyz = p * r[:, None]
    # normals from the mesh itself: average of adjacent cell normals
    nrm = _nodal_normals(xyz, cells)
    return Mesh(xyz, cells, nrm)


def _nodal_normals(xyz, cells):
    v = xyz[cells]
    t1 = (v[:, 1] - v[:, 0]) + (v[:, 3] - v[:, 2])
    t2 = (v[:, 2] - v[:, 0]) + (v[:, 3] - v[:, 1])
    cn = np.cross(t1, t2)
    out = np.zeros_like(xyz)
    for j in range(4):
        np.add.at(out, cells[:, j], cn)
    out /= np.linalg.norm(out, axis=1, keepdims=True)
    return out


def wigley_hull(nx: int, nz: int, ny_lid: int, L=1.0, B=0.1, T=0.0625, lid: bool = True) -> Mesh:
    """Closed Wigley-type hull y = +-(B/2)(1-(2x/L)^2)(1-(z/T)^2), z in [-T,0],
    closed by the lid z = 0.  Port and starboard sides are nx x nz grids, the lid
    an nx x ny_lid grid; the keel (z=-T, y=0) and the bow/stern lines (y=0) are
    single shared node rows.  Outward cell orientation.  lid=False leaves the
    lid out: the wetted surface, open along the waterline z = 0."""
    xs = np.linspace(-L / 2, L / 2, nx + 1)
    zs = np.linspace(-T, 0.0, nz + 1)
    index = {}
    pts = []

    def half_beam(x, z):
        return 0.5 * B * (1 - (2 * x / L) ** 2) * (1 - (z / T) ** 2)

    def node(key, xyz):
        k = index.get(key)
        if k is None:
            k = len(pts)
            index[key] = k
            pts.append(xyz)
        return k

    def side_node(i, j, s):
        x, z = xs[i], zs[j]
        y = s * half_beam(x, z)
        if i == 0 or i == nx or j == 0:  # y == 0 lines shared by both sides
            return node(("c", i, j), [x, 0.0, z])
        if j == nz:  # top edge of a side = a long edge of the lid grid
            return node(("lid", i, ny_lid if s > 0 else 0), [x, y, z])
        return node(("s", i, j, s), [x, y, z])

    cells = []
    for s in (1, -1):
        for j in range(nz):
            for i in range(nx):
                q = [side_node(i, j, s), side_node(i + 1, j, s), side_node(i, j + 1, s),
                     side_node(i + 1, j + 1, s)]
                # starboard (y>0): d/dx x d/dz points -y; flip ordering for outward
                if s > 0:
                    q = [q[0], q[2], q[1], q[3]]
                cells.append(q)
    # lid: z = 0, grid over x and eta in [-1,1] with y = eta * half_beam(x, 0)
    for j in range(ny_lid if lid else 0):
        for i in range(nx):
            quad = []
            for dj in (0, 1):
                for di in (0, 1):
                    ii, jj = i + di, j + dj
                    x = xs[ii]
                    eta = -1.0 + 2.0 * jj / ny_lid
                    y = eta * half_beam(x, 0.0)
                    if ii == 0 or ii == nx:
                        k = node(("c", ii, nz), [x, 0.0, 0.0])
                    elif jj == 0:
                        k = side_node(ii, nz, -1)
                    elif jj == ny_lid:
                        k = side_node(ii, nz, 1)
                    else:
                        k = node(("lid", ii, jj), [x, y, 0.0])
                    quad.append(k)
            cells.append(quad)  # d/dx x d/deta = +z (outward for the lid)
    # The lid cells at the bow and stern keep a collapsed edge (two equal
    # vertices): the surface stays closed and the bilinear map is still
    # regular at the interior quadrature points.
    xyz = np.asarray(pts, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int32)
    return Mesh(xyz, cells, _nodal_normals(xyz, cells))


def point_source_field(sources, strengths):
    """phi(x) = sum_k q_k / |x - s_k| and its gradient."""
    S = np.asarray(sources, dtype=np.float64).reshape(-1, 3)
    q = np.asarray(strengths, dtype=np.float64).reshape(-1)

    def phi(x):
        d = x[:, None, :] - S[None, :, :]
        r = np.linalg.norm(d, axis=2)
        return (q[None, :] / r).sum(axis=1)

    def grad(x):
        d = x[:, None, :] - S[None, :, :]
        r = np.linalg.norm(d, axis=2)
        return -(q[None, :, None] * d / r[:, :, None] ** 3).sum(axis=1)

    return phi, grad


def mixed_bc_by_cell_centroid(mesh: Mesh, z_split: float = 0.0):
    """Dirichlet mask: nodes of cells whose centroid has z > z_split (interface
    nodes are Dirichlet); the rest Neumann."""
    cz = mesh.xyz[mesh.cells][:, :, 2].mean(axis=1)
    mask = np.zeros(mesh.n_nodes, dtype=np.uint8)
    mask[np.unique(mesh.cells[cz > z_split])] = 1
    return mask


def sphere_dirichlet_case(n: int = 16, x0=(2.0, 0.5, 0.3)):
    """Unit cube-sphere, pure Dirichlet phi = 1/|x-x0| (interior problem).

    Returns mesh, dirichlet mask, tmp_rhs (phi at all nodes) and the analytic
    dphi/dn at the nodes."""
    mesh = cube_sphere(n)
    phi, grad = point_source_field([x0], [1.0])
    mask = np.ones(mesh.n_nodes, dtype=np.uint8)
    tmp = phi(mesh.xyz)
    exact_dn = (grad(mesh.xyz) * mesh.normals).sum(axis=1)
    return mesh, mask, tmp, exact_dn


def spheroid_mixed_case(n: int, seed: int, n_sources: int = 8, axes=(3.0, 1.0, 1.0),
                        mesh: Mesh | None = None):
    """Spheroid with mixed data from n_sources point sources of strength U(-1,1)
    uniformly inside |s| < 0.5 (exterior problem).

    Returns mesh, dirichlet mask, tmp_rhs, exact phi, exact dphi/dn."""
    if mesh is None:
        mesh = spheroid(n, axes)
    rng = np.random.Generator(np.random.PCG64(seed))
    q = rng.uniform(-1.0, 1.0, n_sources)
    dirs = rng.normal(size=(n_sources, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rad = 0.5 * rng.uniform(0.0, 1.0, n_sources) ** (1.0 / 3.0)
    S = dirs * rad[:, None]
    phi, grad = point_source_field(S, q)
    mask = mixed_bc_by_cell_centroid(mesh)
    ph = phi(mesh.xyz)
    dn = (grad(mesh.xyz) * mesh.normals).sum(axis=1)
    tmp = np.where(mask == 1, ph, dn)
    return mesh, mask, tmp, ph, dn


def random_plane_mask(mesh: Mesh, seed: int):
    """Dirichlet mask from a seeded random plane: nodes of cells whose centroid
    lies on the positive side are Dirichlet (interface nodes Dirichlet), the
    rest Neumann.  The plane passes within a quarter of the half-extent of the
    mesh centre, so both parts are present."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nrm = rng.normal(size=3)
    nrm /= np.linalg.norm(nrm)
    c = 0.5 * (mesh.xyz.min(axis=0) + mesh.xyz.max(axis=0))
    half = 0.5 * float(np.abs((mesh.xyz - c) @ nrm).max())
    off = rng.uniform(-0.25, 0.25) * half
    cent = mesh.xyz[mesh.cells].mean(axis=1)
    mask = np.zeros(mesh.n_nodes, dtype=np.uint8)
    mask[np.unique(mesh.cells[(cent - c) @ nrm > off])] = 1
    return mask


def sources_in_ball(rng, n_sources: int, radius: float = 0.5):
    """n_sources points uniform in the ball |s| < radius."""
    dirs = rng.normal(size=(n_sources, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rad = radius * rng.uniform(0.0, 1.0, n_sources) ** (1.0 / 3.0)
    return dirs * rad[:, None]


def sources_in_wigley(rng, n_sources: int, L=1.0, B=0.1, T=0.0625):
    """n_sources points inside the Wigley hull, away from its surface:
    |x| < 0.3 L, z in [-0.65 T, -0.35 T], |y| < 0.3 of the local half-beam."""
    x = rng.uniform(-0.3 * L, 0.3 * L, n_sources)
    z = rng.uniform(-0.65 * T, -0.35 * T, n_sources)
    hb = 0.5 * B * (1 - (2 * x / L) ** 2) * (1 - (z / T) ** 2)
    y = rng.uniform(-0.3, 0.3, n_sources) * hb
    return np.stack([x, y, z], axis=1)


def point_source_data(mesh: Mesh, mask, sources, strengths):
    """tmp_rhs (phi on Dirichlet nodes, dphi/dn on Neumann nodes), phi, dphi/dn."""
    phi, grad = point_source_field(sources, strengths)
    ph = phi(mesh.xyz)
    dn = (grad(mesh.xyz) * mesh.normals).sum(axis=1)
    return np.where(mask == 1, ph, dn), ph, dn


def wigley_mixed_case(nx: int, nz: int, ny_lid: int, seed: int = 3, n_sources: int = 8,
                      mesh: Mesh | None = None):
    """Wigley hull with mixed data from n_sources point sources of strength
    U(-1,1) inside the hull (exterior problem): cells with centroid
    z > -T/2 Dirichlet, the rest Neumann.

    Returns mesh, dirichlet mask, tmp_rhs, exact phi, exact dphi/dn."""
    if mesh is None:
        mesh = wigley_hull(nx, nz, ny_lid)
    rng = np.random.Generator(np.random.PCG64(seed))
    q = rng.uniform(-1.0, 1.0, n_sources)
    S = sources_in_wigley(rng, n_sources)
    mask = mixed_bc_by_cell_centroid(mesh, z_split=-0.5 * 0.0625)
    tmp, ph, dn = point_source_data(mesh, mask, S, q)
    return mesh, mask, tmp, ph, dn


def wigley_double_body_case(nx: int, nz: int, seed: int = 5, n_sources: int = 6,
                            z0: float = 0.0):
    """Double body: the wetted Wigley hull (no lid, waterline z = z0 = 0) and
    data from n_sources point sources of strength U(-1,1) inside the hull plus
    their images in the waterline (the field is symmetric about z = z0, so the
    doubled body sees it exactly).  Exterior problem; cells with centroid
    z > -T/2 Dirichlet, the rest Neumann.  Nodal normals on the waterline are
    the horizontal normals of the doubled body.

    Returns mesh, dirichlet mask, tmp_rhs, exact phi, exact dphi/dn."""
    T = 0.0625
    mesh = wigley_hull(nx, nz, 2, lid=False)
    on_plane = np.abs(mesh.xyz[:, 2] - z0) < 1e-12
    nrm = mesh.normals.copy()
    nrm[on_plane, 2] = 0.0
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    mesh = Mesh(mesh.xyz, mesh.cells, nrm)
    rng = np.random.Generator(np.random.PCG64(seed))
    q = rng.uniform(-1.0, 1.0, n_sources)
    S = sources_in_wigley(rng, n_sources)
    Sm = S.copy()
    Sm[:, 2] = 2.0 * z0 - Sm[:, 2]
    mask = mixed_bc_by_cell_centroid(mesh, z_split=-0.5 * T)
    tmp, ph, dn = point_source_data(mesh, mask, np.vstack([S, Sm]), np.concatenate([q, q]))
    return mesh, mask, tmp, ph, dn


def wigley_for_nodes(n_nodes: float) -> tuple[int, int, int]:
    """(nx, nz, ny_lid) in the 6 : 1.5 : 1 proportion of the 768 x 192 + 768 x 128
    hull, for about n_nodes nodes (2 nx nz + nx ny_lid)."""
    nx = max(12, int(round(np.sqrt(1.5 * n_nodes) / 6.0)) * 6)
    return nx, max(3, nx // 4), max(2, nx // 6)


def sphere_n_for_nodes(n_nodes: float) -> int:
    """Cube-sphere resolution n with 6 n^2 + 2 close to n_nodes."""
    return max(2, int(round(np.sqrt(max(n_nodes - 2, 6) / 6.0))))
