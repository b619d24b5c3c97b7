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
