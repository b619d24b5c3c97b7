"""Synthetic inputs for the Kershaw-box Poisson problems (numpy, host side).

The box mesh stands in for the reference's Kershaw benchmark case
(examples/kershaw: genbox box + usrdat vertex map kershaw.usr:107-225).  It is
[0,1]^3 split into nx*ny*nz hexahedra numbered x fastest; vertices are in
hypercube order v = i + 2j + 4k with 1-based lexicographic lattice ids; the
Kershaw map of parameter eps deforms the vertices, so elements stay trilinear.

The right-hand side is f = U[-1,1] per lattice node, i.i.d. from a
counter-based hash (splitmix64 of seed and the global lattice index, so every
copy of a shared node sees the same value), weighted by the lumped mass JW.
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _right(eps, x):
    return np.where(x <= 0.5, (2.0 - eps) * x, 1.0 + eps * (x - 1.0))


def _left(eps, x):
    return 1.0 - _right(eps, 1.0 - x)


def _step(a, b, x):
    return np.where(x <= 0.0, a, np.where(x >= 1.0, b, a + (b - a) * x))


def kershaw_map(eps, x, y, z):
    layer = (x * 6.0).astype(np.int64)
    lam = (x - layer / 6.0) * 6.0
    yy = np.empty_like(y)
    zz = np.empty_like(z)
    m0 = layer == 0
    m14 = (layer == 1) | (layer == 4)
    m2 = layer == 2
    m3 = layer == 3
    m5 = ~(m0 | m14 | m2 | m3)
    for src, out in ((y, yy), (z, zz)):
        L, R = _left(eps, src), _right(eps, src)
        out[m0] = L[m0]
        out[m14] = _step(L, R, lam)[m14]
        out[m2] = _step(R, L, lam / 2.0)[m2]
        out[m3] = _step(R, L, (1.0 + lam) / 2.0)[m3]
        out[m5] = R[m5]
    return x.copy(), yy, zz


def kershaw_box(nx, ny=None, nz=None, eps=0.3, all_dirichlet=True):
    """Return (VX [E,8,3], EToV [E,8] int64, EToB [E,6] int32)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    ex, ey, ez = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ex, ey, ez = (a.transpose(2, 1, 0).ravel() for a in (ex, ey, ez))  # x fastest
    E = nx * ny * nz
    a = np.array([v & 1 for v in range(8)])
    b = np.array([(v >> 1) & 1 for v in range(8)])
    c = np.array([(v >> 2) & 1 for v in range(8)])
    ix = ex[:, None] + a[None, :]
    iy = ey[:, None] + b[None, :]
    iz = ez[:, None] + c[None, :]
    EToV = (1 + ix + (nx + 1) * (iy + (ny + 1) * iz)).astype(np.int64)
    X, Y, Z = kershaw_map(eps, ix / nx, iy / ny, iz / nz)
    VX = np.stack([X, Y, Z], axis=-1).astype(np.float64)
    bc = np.stack([ez == 0, ey == 0, ex == nx - 1, ey == ny - 1, ex == 0, ez == nz - 1], axis=1)
    EToB = np.where(bc, 1 if all_dirichlet else 4, 0).astype(np.int32)
    return VX.reshape(E, 8, 3), EToV, EToB


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def box_lattice_index(N, nx, ny, nz):
    """Global lattice index of every E-vector node of the box mesh."""
    nq = N + 1
    e = np.arange(nx * ny * nz)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    k, j, i = np.meshgrid(np.arange(nq), np.arange(nq), np.arange(nq), indexing="ij")
    gx = ex[:, None] * N + i.ravel()[None, :]
    gy = ey[:, None] * N + j.ravel()[None, :]
    gz = ez[:, None] * N + k.ravel()[None, :]
    Lx, Ly = nx * N + 1, ny * N + 1
    return (gx + Lx * (gy + Ly * gz)).astype(np.uint64).ravel()


def box_field(N, nx, ny, nz, seed):
    """f in U[-1,1], one value per lattice node, as an E-vector."""
    with np.errstate(over="ignore"):
        g = box_lattice_index(N, nx, ny, nz)
        h = _splitmix64(np.uint64(seed) ^ _splitmix64(g))
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


def box_rhs(N, nx, ny, nz, seed, ggeo):
    """Mass-weighted seeded right-hand side: JW * f (E-vector)."""
    Np = (N + 1) ** 3
    E = nx * ny * nz
    JW = np.asarray(ggeo).reshape(E, 7, Np)[:, 6, :].ravel()
    return box_field(N, nx, ny, nz, seed) * JW


def axis_fan(nsec=12, layers=2, radius=1.0, z_bc=1, outer_bc=1):
    """Hexahedra in a fan around the z axis: `nsec` sectors per layer, `layers` layers on [0, layers].

    Sector i of a layer has the corners O (on the axis), A_i, B_i and A_{i+1} (A on the unit circle at
    angle 2 pi i / nsec, B between two A at a larger radius): a convex quadrilateral extruded in z, with r
    along O A_i and s along O A_{i+1}, so the Jacobian is positive.  Every axis edge is shared by `nsec`
    elements and every interior axis vertex by 2 nsec, the conforming case the box meshes do not reach
    (at most four elements per edge, eight per vertex).  Faces between sectors and layers are interior;
    the z = 0 / z = layers faces get `z_bc`, the outer faces `outer_bc` (NRSG_BC_* codes).
    Returns (VX [E,8,3], EToV [E,8] int64, EToB [E,6] int32)."""
    th = 2.0 * np.pi / nsec
    rb = radius / np.cos(th / 2.0) * 1.1
    # vertex ids (1-based): per level z = 0..layers: the axis point, A_0..A_{n-1}, B_0..B_{n-1}
    per = 1 + 2 * nsec

    def vid(level, kind, i):
        return 1 + level * per + (0 if kind == "O" else (1 + i % nsec if kind == "A" else 1 + nsec + i % nsec))

    def xyz(kind, i, z):
        if kind == "O":
            return (0.0, 0.0, z)
        if kind == "A":
            a = th * (i % nsec)
            return (radius * np.cos(a), radius * np.sin(a), z)
        a = th * (i % nsec) + th / 2.0
        return (rb * np.cos(a), rb * np.sin(a), z)

    VX, EToV, EToB = [], [], []
    for lay in range(layers):
        for i in range(nsec):
            quad = [("O", i), ("A", i), ("A", i + 1), ("B", i)]  # (r, s) = (0,0), (1,0), (0,1), (1,1)
            ids, pts = [], []
            for c in range(2):
                for kind, k in quad:
                    ids.append(vid(lay + c, kind, k))
                    pts.append(xyz(kind, k, float(lay + c)))
            VX.append(pts)
            EToV.append(ids)
            # nekRS face order: t=0, s=0, r=1, s=1, r=0, t=1
            EToB.append([z_bc if lay == 0 else 0, 0, outer_bc, outer_bc, 0, z_bc if lay == layers - 1 else 0])
    return (np.array(VX, dtype=np.float64), np.array(EToV, dtype=np.int64), np.array(EToB, dtype=np.int32))
