"""Mesh ingestion from Nek5000 binary ``.re2`` files.

Reading and vertex numbering run in the library's host code (C ABI
``nrsg_re2_*`` / ``nrsg_mesh_connect``, include/nekrs_gb300.h); this module
wraps them and adds the writer (the byte layout of Nek5000's
core/reader_re2.f read in reverse) and a box generator with the element and
corner order of Nek5000's ``genbox``.

    VX, EToV, EToB = mesh_from_re2("kershaw.re2", codes={"O": NRSG_BC_DIRICHLET})
    el = nekrs_gb300.Elliptic(7, VX, EToV, EToB, options)
"""
import ctypes

import numpy as np

from . import LL, check, lib, vp
from . import workloads as W

NRSG_BC_NONE, NRSG_BC_DIRICHLET, NRSG_BC_NEUMANN = 0, 1, 4
# hypercube corner v = i + 2j + 4k  <->  pre-processor corner (self-inverse)
PRE_TO_SYM_VERTEX = np.array([0, 1, 3, 2, 4, 5, 7, 6])
# pre-processor face -> nekRS face (t-, s-, r+, s+, r-, t+)
PRE_TO_NEKRS_FACE = np.array([1, 2, 3, 4, 0, 5])


class Re2Header(ctypes.Structure):
    _fields_ = [("version", ctypes.c_int), ("ndim", ctypes.c_int), ("nelgt", LL), ("nelgv", LL), ("ncurve", LL),
                ("nbcFields", ctypes.c_int), ("byteSwapped", ctypes.c_int)]


def _bind():
    L = lib()
    if getattr(L, "_re2_bound", False):
        return L
    L.nrsg_re2_read_header.argtypes = [ctypes.c_char_p, ctypes.POINTER(Re2Header)]
    L.nrsg_re2_read_elements.argtypes = [ctypes.c_char_p, vp, vp]
    L.nrsg_re2_read_curves.argtypes = [ctypes.c_char_p, vp, vp, vp, vp]
    L.nrsg_re2_read_bc.argtypes = [ctypes.c_char_p, ctypes.c_int, vp, vp]
    L.nrsg_re2_boundary_ids.argtypes = [LL, vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                        ctypes.POINTER(ctypes.c_int), vp]
    L.nrsg_mesh_connect.argtypes = [LL, vp, ctypes.c_double, vp, vp, vp, ctypes.POINTER(LL)]
    L._re2_bound = True
    return L


def read_header(path):
    L = _bind()
    h = Re2Header()
    check(L.nrsg_re2_read_header(str(path).encode(), ctypes.byref(h)))
    return {k: getattr(h, k) for k, _ in Re2Header._fields_}


def read_re2(path, field=0):
    """Everything the file holds: header, corners [E,8,3] (hypercube order), groups [E], boundary codes
    [E,6] (pre-processor face order, 3-character str) and parameters [E,6,5] of section ``field`` (None when
    the file has no boundary section), curved sides."""
    L = _bind()
    p = str(path).encode()
    h = read_header(path)
    E = h["nelgt"]
    VX = np.zeros((E, 8, 3))
    group = np.zeros(E, dtype=np.int32)
    check(L.nrsg_re2_read_elements(p, VX.ctypes.data, group.ctypes.data))
    nc = h["ncurve"]
    curves = {"elem": np.zeros(nc, dtype=np.int64), "face": np.zeros(nc, dtype=np.int32),
              "params": np.zeros((nc, 5)), "type": np.zeros(nc, dtype="S1")}
    if nc:
        check(L.nrsg_re2_read_curves(p, curves["elem"].ctypes.data, curves["face"].ctypes.data,
                                     curves["params"].ctypes.data, curves["type"].ctypes.data))
    cbc = bc = None
    if h["nbcFields"] > 0:
        raw = np.zeros((E, 6, 4), dtype=np.uint8)
        bc = np.zeros((E, 6, 5))
        check(L.nrsg_re2_read_bc(p, field, raw.ctypes.data, bc.ctypes.data))
        cbc = raw[:, :, :3].copy().view("S3")[:, :, 0].astype(str)
        cbc = np.char.ljust(cbc, 3)
    return {"header": h, "VX": VX, "group": group, "cbc": cbc, "bc": bc, "curves": curves}


def _cbc_bytes(cbc):
    a = np.char.ljust(np.asarray(cbc).astype(str), 3)
    out = np.zeros(a.shape + (4,), dtype=np.uint8)
    b = a.astype("S3").view(np.uint8).reshape(a.shape + (3,))
    out[..., :3] = b
    return np.ascontiguousarray(out)


def boundary_ids(cbc, codes):
    """EToB [E,6] in nekRS face order from pre-processor boundary codes, ``codes`` = {code: id}."""
    L = _bind()
    raw = _cbc_bytes(cbc)
    E = raw.shape[0]
    keys = list(codes.keys())
    arr_c = (ctypes.c_char_p * max(1, len(keys)))(*[k.encode() for k in keys])
    arr_i = (ctypes.c_int * max(1, len(keys)))(*[int(codes[k]) for k in keys])
    EToB = np.zeros((E, 6), dtype=np.int32)
    check(L.nrsg_re2_boundary_ids(E, raw.ctypes.data, len(keys), arr_c, arr_i, EToB.ctypes.data))
    return EToB


def connect(VX, tol=0.2, cbc=None, bc=None):
    """Global vertex ids [E,8] (1-based) from corner coordinates, as parCon numbers them on one process;
    faces coded 'P' are matched through ``bc`` (connected element, face)."""
    L = _bind()
    VX = np.ascontiguousarray(VX, dtype=np.float64)
    E = VX.shape[0]
    EToV = np.zeros((E, 8), dtype=np.int64)
    nv = LL(0)
    raw = _cbc_bytes(cbc) if cbc is not None else None
    bcv = np.ascontiguousarray(bc, dtype=np.float64) if bc is not None else None
    check(L.nrsg_mesh_connect(E, VX.ctypes.data, tol, raw.ctypes.data if raw is not None else None,
                              bcv.ctypes.data if bcv is not None else None, EToV.ctypes.data, ctypes.byref(nv)))
    return EToV


def mesh_from_re2(path, codes, field=0, tol=0.2):
    """(VX, EToV, EToB) for nekrs_gb300.Elliptic from a .re2 file; ``codes`` maps boundary codes to boundary
    types (e.g. {"O": NRSG_BC_DIRICHLET, "W": NRSG_BC_NEUMANN}), the role of a case's boundaryTypeMap."""
    m = read_re2(path, field)
    if m["cbc"] is None:
        raise ValueError(f"{path}: no boundary section")
    EToV = connect(m["VX"], tol, m["cbc"], m["bc"])
    return m["VX"], EToV, boundary_ids(m["cbc"], codes)


def kershaw_mesh_from_re2(path, eps, codes=None, field=0, tol=0.2):
    """The Kershaw benchmark mesh from a box .re2 (e.g. the reference case's kershaw.re2): corners rescaled to
    [0, 1]^3 and moved by the Kershaw map of parameter ``eps``; 'O' faces Dirichlet unless ``codes`` says
    otherwise (kershaw.usr:90-95 sets boundary id 1 on them)."""
    VX, EToV, EToB = mesh_from_re2(path, codes or {"O": NRSG_BC_DIRICHLET}, field, tol)
    P = VX.reshape(-1, 3)
    lo, hi = P.min(0), P.max(0)
    U = (VX - lo) / (hi - lo)
    X, Y, Z = W.kershaw_map(eps, U[..., 0], U[..., 1], U[..., 2])
    return np.stack([X, Y, Z], axis=-1), EToV, EToB


def write_re2(path, VX, cbc=None, bc=None, group=None, curves=None, version=2, nelgv=None, byteorder="<",
              extra_bc=()):
    """Write a .re2 file: corners [E,8,3] in hypercube order, boundary codes [E,6] in pre-processor face order
    ('E  ' or '' for none) with parameters [E,6,5]; ``extra_bc`` adds further boundary sections (list of
    (cbc, bc)); ``curves`` = dict(elem, face (0-based), params [n,5], type)."""
    VX = np.asarray(VX, dtype=np.float64)
    E = VX.shape[0]
    nelgv = E if nelgv is None else nelgv
    sections = [] if cbc is None else [(cbc, bc)]
    sections += list(extra_bc)
    if version == 4:
        hdr = f"#v004 {E} 3 {nelgv} {len(sections)} hdr"
    elif version in (2, 3):
        hdr = f"#v00{version}{E:9d}{3:3d}{nelgv:9d} hdr"
    else:
        raise ValueError("version must be 2, 3 or 4")
    f8 = np.dtype(byteorder + "f8")
    out = [hdr.ljust(80).encode(), np.array([6.54321], dtype=byteorder + "f4").tobytes()]
    rec = np.zeros((E, 25), dtype=f8)
    rec[:, 0] = 0 if group is None else np.asarray(group)
    pre = VX[:, PRE_TO_SYM_VERTEX, :]
    rec[:, 1:9], rec[:, 9:17], rec[:, 17:25] = pre[:, :, 0], pre[:, :, 1], pre[:, :, 2]
    out.append(rec.tobytes())

    def records(elem, face, params, codes):
        n = len(elem)
        r = np.zeros(n, dtype=np.dtype([("w", f8, 7), ("c", "S8")]))
        r["w"][:, 0] = np.asarray(elem) + 1
        r["w"][:, 1] = np.asarray(face) + 1
        r["w"][:, 2:] = params
        r["c"] = [c.encode().ljust(8) for c in codes]
        return np.array([n], dtype=f8).tobytes() + r.tobytes()

    if curves is None:
        out.append(records([], [], np.zeros((0, 5)), []))
    else:
        out.append(records(curves["elem"], curves["face"], curves["params"],
                           [t.decode() if isinstance(t, bytes) else str(t) for t in curves["type"]]))
    for c, b in sections:
        c = np.char.ljust(np.asarray(c).astype(str), 3)
        b = np.zeros((E, 6, 5)) if b is None else np.asarray(b, dtype=np.float64)
        sel = np.argwhere((c != "E  ") & (c != "   "))  # element order, then face
        out.append(records(sel[:, 0], sel[:, 1], b[sel[:, 0], sel[:, 1]], [c[e, f] for e, f in sel]))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


def box(nx, ny, nz, xs, ys, zs, sides=("E",) * 6):
    """Box mesh in genbox's layout: element e = ix + nx*(iy + ny*iz), corners at the lattice values xs[ix..ix+1]
    etc.  ``sides`` = boundary codes of the (x-, x+, y-, y+, z-, z+) sides.  Returns (VX [E,8,3] hypercube
    order, cbc [E,6] pre-processor face order)."""
    xs, ys, zs = (np.asarray(a, dtype=np.float64) for a in (xs, ys, zs))
    e = np.arange(nx * ny * nz)
    ix, iy, iz = e % nx, (e // nx) % ny, e // (nx * ny)
    v = np.arange(8)
    a, b, c = v & 1, (v >> 1) & 1, (v >> 2) & 1
    VX = np.stack([xs[ix[:, None] + a], ys[iy[:, None] + b], zs[iz[:, None] + c]], axis=-1)
    cbc = np.full((nx * ny * nz, 6), "E  ", dtype="<U3")
    # pre-processor faces: 0 s-, 1 r+, 2 s+, 3 r-, 4 t-, 5 t+
    for face, side, cond in ((0, 2, iy == 0), (1, 1, ix == nx - 1), (2, 3, iy == ny - 1), (3, 0, ix == 0),
                             (4, 4, iz == 0), (5, 5, iz == nz - 1)):
        cbc[cond, face] = sides[side].ljust(3)
    return VX, cbc
