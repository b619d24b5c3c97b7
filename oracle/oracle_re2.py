"""Oracle (test infrastructure only): numpy restatement of the .re2 reader and
of parCon's vertex numbering, used by tests/ to check the library's host code.

Reader: Nek5000 core/reader_re2.f (read_re2_hdr :543-620, readp_re2_mesh
:68-157, readp_re2_curve :159-286, readp_re2_bc :288-428), 8-byte words.
Numbering: parRSB parrsb_conn_mesh (con.c:221-321) on one process --
findMinNeighborDistance (con.c:85-117), find_unique_vertices
(con-unique-vertices.c:385-446: ndim rounds of per-segment sorts by x, y, z
with the split test of find_segments :237-257), setGlobalID (con.c:123-155),
matchPeriodicFaces (con-periodic.c:266-281) with findConnectedPeriodicPairs
(:117-178) and compressPeriodicVertices (:17-50).
"""
import numpy as np

PRE_TO_SYM_VERTEX = np.array([0, 1, 3, 2, 4, 5, 7, 6])
PRE_TO_SYM_FACE = np.array([2, 1, 3, 0, 4, 5])
NEIGHBOR = np.array([[1, 2, 4], [0, 3, 5], [0, 3, 6], [1, 2, 7], [0, 5, 6], [1, 4, 7], [2, 4, 7], [3, 5, 6]])
SYM_FACE_VERTS = np.array([[1, 5, 7, 3], [2, 4, 8, 6], [1, 2, 6, 5], [3, 7, 8, 4], [1, 3, 4, 2], [5, 6, 8, 7]]) - 1


def read(path):
    b = open(path, "rb").read()
    hdr = b[:80].decode()
    ver = hdr[:5]
    if ver == "#v004":
        t = hdr[5:].split()
        nelgt, ndim, nelgv = int(t[0]), int(t[1]), int(t[2])
    else:
        nelgt, ndim, nelgv = int(hdr[5:14]), int(hdr[14:17]), int(hdr[17:26])
    bo = "<" if np.frombuffer(b[80:84], "<f4")[0] == np.float32(6.54321) else ">"
    f8 = np.dtype(bo + "f8")
    off = 84
    el = np.frombuffer(b[off:off + nelgt * 200], f8).reshape(nelgt, 25)
    off += nelgt * 200
    pre = np.stack([el[:, 1:9], el[:, 9:17], el[:, 17:25]], axis=-1)
    VX = pre[:, PRE_TO_SYM_VERTEX, :].astype(np.float64)
    rec_t = np.dtype([("w", f8, 7), ("c", "S8")])

    def section(off):
        n = int(np.frombuffer(b[off:off + 8], f8)[0])
        r = np.frombuffer(b[off + 8:off + 8 + 64 * n], rec_t)
        return r, off + 8 + 64 * n

    curves, off = section(off)
    bcs = []
    while off < len(b):
        r, off = section(off)
        cbc = np.full((nelgt, 6), "E  ", dtype="<U3")
        bc = np.zeros((nelgt, 6, 5))
        e = r["w"][:, 0].astype(np.int64) - 1
        f = r["w"][:, 1].astype(np.int64) - 1
        cbc[e, f] = [c[:3].decode() for c in r["c"]]
        bc[e, f] = r["w"][:, 2:]
        bcs.append((cbc, bc))
    return {"version": int(ver[2:]), "nelgt": nelgt, "nelgv": nelgv, "ndim": ndim, "VX": VX,
            "group": el[:, 0].astype(np.int32), "curves": curves, "bcs": bcs}


def connect(VX, tol=0.2, cbc=None, bc=None):
    VX = np.asarray(VX, dtype=np.float64)
    E = VX.shape[0]
    pts = VX.reshape(E * 8, 3)
    nb = VX[:, NEIGHBOR, :]  # [E,8,3,3]
    dx = (((VX[:, :, None, :] - nb) ** 2).sum(-1)).min(-1).reshape(-1)
    order = np.arange(E * 8)
    start = np.zeros(E * 8, dtype=bool)
    start[0] = True
    tol2 = tol * tol
    for _t in range(3):
        for d in range(3):
            bounds = np.flatnonzero(start).tolist() + [E * 8]
            for s, e in zip(bounds[:-1], bounds[1:]):
                if e - s > 1:
                    seg = order[s:e]
                    order[s:e] = seg[np.argsort(pts[seg, d], kind="stable")]
            xd = pts[order, d]
            m = np.minimum(dx[order][1:], dx[order][:-1]) * tol2
            start[1:] |= (xd[1:] - xd[:-1]) ** 2 > m
    seg_id = np.cumsum(start) - 1
    gid = np.empty(E * 8, dtype=np.int64)
    gid[order] = seg_id
    if cbc is not None:
        faces = []
        for e in range(E):
            for f in range(6):
                if str(cbc[e][f]).startswith("P"):
                    faces.append((e, PRE_TO_SYM_FACE[f], int(bc[e][f][0]) - 1, PRE_TO_SYM_FACE[int(bc[e][f][1]) - 1]))
        root = np.arange(E * 8)

        def find(a):
            while root[a] != a:
                a = root[a]
            return a

        for i in range(len(faces)):
            for j in range(i + 1, len(faces)):
                ei, fi = faces[i][0], faces[i][1]
                ej, fj, cej, cfj = faces[j]
                if not (cej == ei and cfj == fi):
                    continue
                pf = ei * 8 + SYM_FACE_VERTS[fi]
                pg = ej * 8 + SYM_FACE_VERTS[fj]
                xf, xg = pts[pf].copy(), pts[pg].copy()
                fmax, gmax = np.abs(xf).max(), np.abs(xg).max()
                xf -= xf.mean(0)
                xg -= xg.mean(0)
                best, shift = 1e20, 0
                for s in range(4):
                    k = 3 - (np.arange(4) + s) % 4
                    d2 = ((xf - xg[k]) ** 2).sum()
                    if d2 < best:
                        best, shift = d2, s
                assert np.sqrt(best) <= 1e-3 * max(fmax, gmax), "periodic faces do not match"
                k = 3 - (np.arange(4) + shift) % 4
                for a, b2 in zip(gid[pf], gid[pg[k]]):
                    ra, rb = find(a), find(b2)
                    if ra != rb:
                        root[max(ra, rb)] = min(ra, rb)
        gid = np.array([find(g) for g in gid])
    _, comp = np.unique(gid, return_inverse=True)
    return (comp + 1).reshape(E, 8).astype(np.int64)
