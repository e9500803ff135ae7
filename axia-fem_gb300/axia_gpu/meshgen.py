"""Seeded synthetic structured hexahedral meshes and load cases.

The reference solves INP decks; the workloads here are the same models built
programmatically: structured C3D8 / C3D20 blocks with CalculiX node order
(solver/src/elem.rs:147-156 HEX_XI, solver/src/quadratic.rs:13-34 HEX20_XI),
single-point constraints as full-DOF indices (dof = 3*node + direction,
solver/src/analysis.rs:152-154) and loads as CLOAD entries or DLOAD face
pressures (face ids P1..P6 as in solver/src/elem.rs:894-901).

All randomness comes from numpy's PCG64 seeded generator, so a seed gives the
same mesh on every machine.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

# (xi, eta, zeta) of the 20 C3D20 nodes in CalculiX order; the first 8 are the
# C3D8 nodes (solver/src/quadratic.rs:13-34).
HEX20_XI = np.array(
    [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
     [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1],
     [0, -1, -1], [1, 0, -1], [0, 1, -1], [-1, 0, -1],
     [0, -1, 1], [1, 0, 1], [0, 1, 1], [-1, 0, 1],
     [-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], dtype=np.int64)

# Face ids of a hexahedron (1-based, CalculiX P1..P6) by outward direction.
FACE_ZMIN, FACE_ZMAX, FACE_YMIN, FACE_XMAX, FACE_YMAX, FACE_XMIN = 1, 2, 3, 4, 5, 6


@dataclass
class Model:
    """A C3D8 / C3D20 linear-static model in the arrays the C ABI takes."""

    name: str
    coords: np.ndarray          # (n_nodes, 3) float64
    conn: np.ndarray            # (n_elem, nn) int32, 0-based node indices
    nn: int                     # 8 or 20
    e_elem: np.ndarray          # (n_elem,) float64 Young's modulus
    nu: float
    bc_dof: np.ndarray          # (n_bc,) int64 full DOF index; later entries win
    bc_val: np.ndarray          # (n_bc,) float64 prescribed value
    cload: np.ndarray           # (3*n_nodes,) float64 concentrated nodal loads
    dload_elem: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    dload_face: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    dload_p: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    reduced: bool = False       # C3D20R (2x2x2 Gauss)
    shape: tuple = ()

    @property
    def n_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_elem(self) -> int:
        return int(self.conn.shape[0])

    @property
    def ndof(self) -> int:
        return 3 * self.n_nodes

    def free_mask(self) -> np.ndarray:
        m = np.ones(self.ndof, dtype=bool)
        m[self.bc_dof] = False
        return m

    @property
    def n_free(self) -> int:
        return int(self.free_mask().sum())


def _grid_c3d8(nx, ny, nz, h):
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    # node id = i + (nx+1)*(j + (ny+1)*k): x fastest
    coords = np.empty(((nx + 1) * (ny + 1) * (nz + 1), 3))
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    ids = nid(ii, jj, kk).ravel()
    coords[ids, 0] = (ii.ravel()) * h
    coords[ids, 1] = (jj.ravel()) * h
    coords[ids, 2] = (kk.ravel()) * h
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    eid = (ei + nx * (ej + ny * ek)).ravel()
    conn = np.empty((nx * ny * nz, 8), dtype=np.int32)
    for a in range(8):
        dx = (HEX20_XI[a, 0] + 1) // 2
        dy = (HEX20_XI[a, 1] + 1) // 2
        dz = (HEX20_XI[a, 2] + 1) // 2
        conn[eid, a] = nid(ei + dx, ej + dy, ek + dz).ravel()
    lattice = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1)
    lat = np.empty_like(lattice)
    lat[ids] = lattice
    return coords, conn, lat


def _grid_c3d20(nx, ny, nz, h):
    """Nodes on the half-step lattice with at most one odd index."""
    mx, my, mz = 2 * nx + 1, 2 * ny + 1, 2 * nz + 1
    gi, gj, gk = np.meshgrid(np.arange(mx), np.arange(my), np.arange(mz), indexing="ij")
    # lexicographic order with x fastest
    gi = gi.transpose(2, 1, 0).ravel()
    gj = gj.transpose(2, 1, 0).ravel()
    gk = gk.transpose(2, 1, 0).ravel()
    keep = ((gi & 1) + (gj & 1) + (gk & 1)) <= 1
    node_of = np.full(mx * my * mz, -1, dtype=np.int64)
    node_of[keep] = np.arange(int(keep.sum()))
    coords = np.stack([gi[keep], gj[keep], gk[keep]], axis=1).astype(np.float64) * (0.5 * h)
    lat = np.stack([gi[keep], gj[keep], gk[keep]], axis=1)
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    eid = (ei + nx * (ej + ny * ek)).ravel()
    conn = np.empty((nx * ny * nz, 20), dtype=np.int32)
    for a in range(20):
        li = 2 * ei + HEX20_XI[a, 0] + 1
        lj = 2 * ej + HEX20_XI[a, 1] + 1
        lk = 2 * ek + HEX20_XI[a, 2] + 1
        conn[eid, a] = node_of[(li + mx * (lj + my * lk)).ravel()]
    assert (conn >= 0).all()
    return coords, conn, lat


def structured_block(nx, ny, nz, nn=8, h=1.0):
    """coords, conn and the integer lattice position of each node (half steps for C3D20)."""
    if nn == 8:
        return _grid_c3d8(nx, ny, nz, h)
    if nn == 20:
        return _grid_c3d20(nx, ny, nz, h)
    raise ValueError("nn must be 8 or 20")


def _clamp_dofs(node_mask):
    nodes = np.nonzero(node_mask)[0].astype(np.int64)
    return (3 * nodes[:, None] + np.arange(3)[None, :]).ravel()


def cantilever_c3d8(nx=20, ny=4, nz=4, h=1.0, e=210000.0, nu=0.3, fz_total=-1000.0):
    """C3D8 cantilever of h-sized cubes: x=0 fully fixed, Fz split evenly over the x=L nodes."""
    coords, conn, lat = structured_block(nx, ny, nz, 8, h)
    clamp = lat[:, 0] == 0
    tip = np.nonzero(lat[:, 0] == nx)[0]
    f = np.zeros(3 * coords.shape[0])
    f[3 * tip + 2] = fz_total / len(tip)
    bc = _clamp_dofs(clamp)
    return Model(f"c3d8_cantilever_{nx}x{ny}x{nz}", coords, conn, 8, np.full(conn.shape[0], e), nu,
                 bc, np.zeros(bc.shape[0]), f, shape=(nx, ny, nz))


def perturb_interior(coords, lat, lat_max, amp, h, seed):
    """Moves every node off the outer boundary by U(-amp, amp)*h per coordinate."""
    rng = np.random.default_rng(seed)
    interior = np.all((lat > 0) & (lat < np.asarray(lat_max)[None, :]), axis=1)
    d = rng.uniform(-amp, amp, size=(int(interior.sum()), 3)) * h
    out = coords.copy()
    out[interior] += d
    return out


def block_c3d8_pressure(n=100, h=1.0, e=210000.0, nu=0.3, p=1.0, perturb=0.15, seed=20261203):
    """C3D8 n^3 block: x=0 clamped, uniform pressure p on x=L (face P4), interior nodes perturbed."""
    coords, conn, lat = structured_block(n, n, n, 8, h)
    if perturb > 0:
        coords = perturb_interior(coords, lat, (n, n, n), perturb, h, seed)
    bc = _clamp_dofs(lat[:, 0] == 0)
    eids = np.arange(conn.shape[0], dtype=np.int64)
    ex = eids % n
    le = eids[ex == n - 1]
    return Model(f"c3d8_block_{n}^3", coords, conn, 8, np.full(conn.shape[0], e), nu, bc,
                 np.zeros(bc.shape[0]), np.zeros(3 * coords.shape[0]),
                 le, np.full(le.shape[0], FACE_XMAX, np.int32), np.full(le.shape[0], p), shape=(n, n, n))


def block_c3d20_traction(n=50, h=1.0, e=70000.0, nu=0.33, seed=20261203, reduced=False):
    """C3D20 n^3 block: base z=0 clamped, per-element top-face (P2) pressure ~ N(0,1) MPa."""
    coords, conn, lat = structured_block(n, n, n, 20, h)
    bc = _clamp_dofs(lat[:, 2] == 0)
    rng = np.random.default_rng(seed)
    eids = np.arange(conn.shape[0], dtype=np.int64)
    top = eids[eids // (n * n) == n - 1]
    p = rng.standard_normal(top.shape[0])
    return Model(f"c3d20_block_{n}^3", coords, conn, 20, np.full(conn.shape[0], e), nu, bc,
                 np.zeros(bc.shape[0]), np.zeros(3 * coords.shape[0]),
                 top, np.full(top.shape[0], FACE_ZMAX, np.int32), p, reduced=reduced, shape=(n, n, n))


def surface_nodes(lat, lat_max):
    lm = np.asarray(lat_max)[None, :]
    return np.nonzero(np.any((lat == 0) | (lat == lm), axis=1))[0]


def random_surface_loads(n_nodes, lat, lat_max, nrhs, frac=0.05, seed=20261203):
    """nrhs nodal force fields: each picks frac of the surface nodes, 3 components ~ N(0,1) N."""
    surf = surface_nodes(lat, lat_max)
    k = max(1, int(round(frac * surf.shape[0])))
    f = np.zeros((nrhs, 3 * n_nodes))
    for r in range(nrhs):
        rng = np.random.default_rng([seed, r])
        pick = rng.choice(surf, size=k, replace=False)
        vals = rng.standard_normal((k, 3))
        idx = 3 * pick[:, None] + np.arange(3)[None, :]
        f[r, idx.ravel()] = vals.ravel()
    return f


def block_c3d8_multiload(n=80, nrhs=32, h=1.0, e=210000.0, nu=0.3, seed=20261203):
    """C3D8 n^3 block, x=0 clamped, with nrhs random surface force fields (rows of .cload_batch)."""
    coords, conn, lat = structured_block(n, n, n, 8, h)
    bc = _clamp_dofs(lat[:, 0] == 0)
    fb = random_surface_loads(coords.shape[0], lat, (n, n, n), nrhs, seed=seed)
    m = Model(f"c3d8_block_{n}^3_x{nrhs}", coords, conn, 8, np.full(conn.shape[0], e), nu, bc,
              np.zeros(bc.shape[0]), fb[0].copy(), shape=(n, n, n))
    m.cload_batch = fb
    return m


def cube_family(count=64, lo=10, hi=40, seed=20261203, e=210000.0, nu=0.3):
    """count independent C3D8 cubes with edge counts ~ U{lo..hi}, x=0 clamped, random surface load."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, size=count)
    out = []
    for i, n in enumerate(sizes):
        coords, conn, lat = structured_block(int(n), int(n), int(n), 8, 1.0)
        bc = _clamp_dofs(lat[:, 0] == 0)
        f = random_surface_loads(coords.shape[0], lat, (n, n, n), 1, seed=seed + 1 + i)[0]
        out.append(Model(f"c3d8_cube_{n}", coords, conn, 8, np.full(conn.shape[0], e), nu, bc,
                         np.zeros(bc.shape[0]), f, shape=(int(n),) * 3))
    return out


def simp_beam(nx=100, ny=50, nz=50, e0=1.0, nu=0.3, pexp=3.0, seed=20261203):
    """C3D8 beam, E_e = E0 rho_e^p with rho_e ~ U[0.3, 1], x=0 clamped, unit -z load at the tip mid-node."""
    coords, conn, lat = structured_block(nx, ny, nz, 8, 1.0)
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.3, 1.0, size=conn.shape[0])
    bc = _clamp_dofs(lat[:, 0] == 0)
    tip = np.nonzero((lat[:, 0] == nx) & (lat[:, 1] == ny // 2) & (lat[:, 2] == nz // 2))[0]
    f = np.zeros(3 * coords.shape[0])
    f[3 * tip[0] + 2] = -1.0
    m = Model(f"c3d8_simp_{nx}x{ny}x{nz}", coords, conn, 8, e0 * rho ** pexp, nu, bc,
              np.zeros(bc.shape[0]), f, shape=(nx, ny, nz))
    m.rho = rho
    m.pexp = pexp
    m.e0 = e0
    return m


def patch_c3d8():
    """One 10 mm C3D8 cube under uniaxial tension: 4 x 5250 N on the x=10 face.

    Same model as the reference's C3D8 patch test (solver/src/lib.rs:234-274,
    examples/patch_c3d8.inp): node 1,4,5,8 fixed in x, node 1 in y and z,
    node 4 in z.  Expected mean u_x on the loaded face: FL/EA = 0.01.
    """
    coords = np.array([[0, 0, 0], [10, 0, 0], [10, 10, 0], [0, 10, 0],
                       [0, 0, 10], [10, 0, 10], [10, 10, 10], [0, 10, 10]], dtype=np.float64)
    conn = np.arange(8, dtype=np.int32)[None, :]
    bcs = [(n, 0) for n in (0, 3, 4, 7)] + [(0, 1), (0, 2), (3, 2)]
    bc = np.array([3 * n + d for n, d in bcs], dtype=np.int64)
    f = np.zeros(24)
    for n in (1, 2, 5, 6):
        f[3 * n] = 5250.0
    return Model("patch_c3d8", coords, conn, 8, np.array([210000.0]), 0.3, bc, np.zeros(bc.shape[0]), f)


def patch_c3d20():
    """One 10 mm C3D20 cube, pressure 210 on face P4 (x=10), positive = compression.

    Same model as the reference's C3D20 patch test (solver/src/lib.rs:700-773):
    nodes 1,4,5,8,12,16,17,20 fixed in x, node 1 in y and z, node 4 in z.
    Expected mean u_x of the corner nodes 2,3,6,7: -0.01.
    """
    coords = np.array([[0, 0, 0], [10, 0, 0], [10, 10, 0], [0, 10, 0],
                       [0, 0, 10], [10, 0, 10], [10, 10, 10], [0, 10, 10],
                       [5, 0, 0], [10, 5, 0], [5, 10, 0], [0, 5, 0],
                       [5, 0, 10], [10, 5, 10], [5, 10, 10], [0, 5, 10],
                       [0, 0, 5], [10, 0, 5], [10, 10, 5], [0, 10, 5]], dtype=np.float64)
    conn = np.arange(20, dtype=np.int32)[None, :]
    fixed_x = [1, 4, 5, 8, 12, 16, 17, 20]
    bcs = [(n - 1, 0) for n in fixed_x] + [(0, 1), (0, 2), (3, 2)]
    bc = np.array([3 * n + d for n, d in bcs], dtype=np.int64)
    return Model("patch_c3d20", coords, conn, 20, np.array([210000.0]), 0.3, bc, np.zeros(bc.shape[0]),
                 np.zeros(60), np.array([0], np.int64), np.array([FACE_XMAX], np.int32), np.array([210.0]))


def from_fixture(path):
    """A model from a JSON fixture with the fields of Model (tests/golden/le10_*.json:
    coords, 0-based conn, e, nu, bc_dof, bc_val, dload_elem/face/p)."""
    import json
    d = json.load(open(path))
    coords = np.array(d["coords"], dtype=np.float64)
    conn = np.array(d["conn"], dtype=np.int32)
    nn = conn.shape[1]
    m = Model(os.path.splitext(os.path.basename(path))[0], coords, conn, nn,
              np.full(conn.shape[0], float(d["e"])), float(d["nu"]),
              np.array(d["bc_dof"], np.int64), np.array(d["bc_val"], np.float64), np.zeros(3 * coords.shape[0]),
              np.array(d["dload_elem"], np.int64), np.array(d["dload_face"], np.int32),
              np.array(d["dload_p"], np.float64))
    m.node_d = int(d.get("node_d", -1))
    return m


# Corner order of the six tetrahedra of a cube split along its main diagonal
# (Kuhn subdivision): tet = (v000, v000 + e_a, v000 + e_a + e_b, v111) for the six
# axis orders (a, b, c); odd orders are listed with two nodes swapped so every
# tetrahedron has a positive Jacobian (elem.rs:221-231 node order).
_KUHN = [((0, 1, 2), False), ((0, 2, 1), True), ((1, 0, 2), True), ((1, 2, 0), False),
         ((2, 0, 1), False), ((2, 1, 0), True)]
# midside nodes of C3D10 in CalculiX order: edges 0-1, 1-2, 2-0, 0-3, 1-3, 2-3
TET10_EDGES = [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]


def structured_tets(nx, ny, nz, nn=4, h=1.0):
    """coords, conn (C3D4 or C3D10, 6 tets per cube) and the doubled lattice position of each node."""
    cells = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    corners = []
    for order, swap in _KUHN:
        v = [np.zeros(3, np.int64)]
        for ax in order:
            step = v[-1].copy()
            step[ax] += 1
            v.append(step)
        t = [v[0], v[1], v[2], v[3]]
        if swap:
            t[1], t[2] = t[2], t[1]
        corners.append(np.stack(t))
    corners = np.stack(corners)                            # (6, 4, 3) unit-cube offsets
    tet = (2 * (cells[:, None, None, :] + corners[None])).reshape(-1, 4, 3)  # doubled lattice
    pts = [tet[:, a] for a in range(4)]
    if nn == 10:
        pts += [(tet[:, a] + tet[:, b]) // 2 for a, b in TET10_EDGES]
    allp = np.stack(pts, axis=1)                           # (n_tet, nn, 3)
    mx, my = 2 * nx + 1, 2 * ny + 1
    key = allp[..., 0] + mx * (allp[..., 1] + my * allp[..., 2])
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    conn = inv.reshape(key.shape).astype(np.int32)
    lat = np.stack([uniq % mx, (uniq // mx) % my, uniq // (mx * my)], axis=1)
    coords = lat.astype(np.float64) * (0.5 * h)
    return coords, conn, lat


def block_tet(n=6, nn=4, h=1.0, e=210000.0, nu=0.3, fx_total=1000.0, perturb=0.0, seed=7):
    """C3D4 / C3D10 n^3 cube block (6 tets per cube): x=0 clamped, a total force fx_total
    split evenly over the x=L nodes (the reference applies no face pressure to tetrahedra,
    analysis.rs:1447), interior nodes optionally perturbed."""
    coords, conn, lat = structured_tets(n, n, n, nn, h)
    if perturb > 0:
        coords = perturb_interior(coords, lat, (2 * n, 2 * n, 2 * n), perturb, 0.5 * h, seed)
    bc = _clamp_dofs(lat[:, 0] == 0)
    tip = np.nonzero(lat[:, 0] == 2 * n)[0]
    f = np.zeros(3 * coords.shape[0])
    f[3 * tip] = fx_total / len(tip)
    return Model(f"c3d{nn}_block_{n}", coords, conn, nn, np.full(conn.shape[0], e), nu, bc, np.zeros(bc.shape[0]),
                 f, shape=(n, n, n))


# Wedges: each cube cell is cut along its xy diagonal into two triangular prisms
# extruded in z.  Corner order (solver/src/extra.rs:84-107): bottom triangle
# (0, 1, 2) at zeta = -1 with (x0 - x2) x (x1 - x2) pointing to the top face,
# then the top triangle (3, 4, 5); C3D15 adds mid-sides 6..8 (bottom edges 0-1,
# 1-2, 2-0), 9..11 (top edges) and 12..14 (vertical edges 0-3, 1-4, 2-5).
_WEDGE_TRI = [((1, 0), (1, 1), (0, 0)), ((1, 1), (0, 1), (0, 0))]
WEDGE15_EDGES = [(0, 1), (1, 2), (2, 0), (3, 4), (4, 5), (5, 3), (0, 3), (1, 4), (2, 5)]


def structured_wedges(nx, ny, nz, nn=6, h=1.0):
    """coords, conn (C3D6 or C3D15, 2 wedges per cube) and the doubled lattice position of each node."""
    cells = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    corners = []
    for tri in _WEDGE_TRI:
        bot = [(a, b, 0) for a, b in tri]
        top = [(a, b, 1) for a, b in tri]
        corners.append(np.array(bot + top, np.int64))
    corners = np.stack(corners)                            # (2, 6, 3) unit-cube offsets
    wed = (2 * (cells[:, None, None, :] + corners[None])).reshape(-1, 6, 3)
    pts = [wed[:, a] for a in range(6)]
    if nn == 15:
        pts += [(wed[:, a] + wed[:, b]) // 2 for a, b in WEDGE15_EDGES]
    allp = np.stack(pts, axis=1)
    mx, my = 2 * nx + 1, 2 * ny + 1
    key = allp[..., 0] + mx * (allp[..., 1] + my * allp[..., 2])
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    conn = inv.reshape(key.shape).astype(np.int32)
    lat = np.stack([uniq % mx, (uniq // mx) % my, uniq // (mx * my)], axis=1)
    coords = lat.astype(np.float64) * (0.5 * h)
    return coords, conn, lat


def block_wedge(n=6, nn=6, h=1.0, e=210000.0, nu=0.3, p=10.0, perturb=0.0, seed=7):
    """C3D6 / C3D15 n^3 cube block (2 wedges per cube): x=0 clamped, pressure p on the
    x=L faces (face P3 = nodes 0-1-4-3 of the first wedge of each cell lies on x = 1
    of the cell; the traction -p n_out pushes inward), interior nodes optionally perturbed."""
    coords, conn, lat = structured_wedges(n, n, n, nn, h)
    if perturb > 0:
        coords = perturb_interior(coords, lat, (2 * n, 2 * n, 2 * n), perturb, 0.5 * h, seed)
    bc = _clamp_dofs(lat[:, 0] == 0)
    cell_x = np.arange(conn.shape[0]) // 2 // (n * n)      # cells are ordered x-major
    loaded = np.nonzero((cell_x == n - 1) & (np.arange(conn.shape[0]) % 2 == 0))[0]
    m = Model(f"c3d{nn}_block_{n}", coords, conn, nn, np.full(conn.shape[0], e), nu, bc, np.zeros(bc.shape[0]),
              np.zeros(3 * coords.shape[0]), loaded.astype(np.int64), np.full(loaded.shape[0], 3, np.int32),
              np.full(loaded.shape[0], p), shape=(n, n, n))
    return m
