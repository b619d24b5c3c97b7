"""Mesh ingestion (.re2 reader, writer, parCon vertex numbering): host code of
the library against the reference's own Kershaw mesh file (pinned through
tests/golden/re2_kershaw.json) and against the oracle's numpy restatement."""
import hashlib
import json
import os

import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import re2 as R
from nekrs_gb300 import workloads as W
from oracle import oracle_re2 as OR

GOLD = os.path.join(os.path.dirname(__file__), "golden", "re2_kershaw.json")


@pytest.fixture(scope="module")
def gold():
    return json.load(open(GOLD))


@pytest.fixture(scope="module")
def kershaw_file(tmp_path_factory, gold):
    """The reference's kershaw.re2, rebuilt from the fixture's lattice by the library's writer."""
    lat = [np.array([float.fromhex(h) for h in a]) for a in gold["lattice_hex"]]
    nx, ny, nz = gold["box"]
    VX, cbc = R.box(nx, ny, nz, lat[0], lat[1], lat[2], (gold["bc_codes"][0].strip(),) * 6)
    p = tmp_path_factory.mktemp("re2") / "kershaw.re2"
    R.write_re2(p, VX, cbc)
    return p, VX, cbc, lat


def test_writer_rebuilds_reference_file_bit_for_bit(product_lib, gold, kershaw_file):
    p = kershaw_file[0]
    b = open(p, "rb").read()
    assert len(b) == gold["bytes"]
    assert b[:80].decode() == gold["header"]
    assert hashlib.sha256(b).hexdigest() == gold["sha256"]


def test_reader_matches_oracle_and_fixture(product_lib, gold, kershaw_file):
    p, VX, cbc, lat = kershaw_file
    m = R.read_re2(p)
    o = OR.read(p)
    h = m["header"]
    assert (h["version"], h["nelgt"], h["nelgv"], h["ncurve"], h["nbcFields"], h["byteSwapped"]) == \
        (2, gold["nelgt"], gold["nelgt"], gold["ncurve"], 1, 0)
    assert np.array_equal(m["VX"], o["VX"]) and np.array_equal(m["VX"], VX)
    assert np.array_equal(m["cbc"], o["bcs"][0][0]) and np.array_equal(m["bc"], o["bcs"][0][1])
    assert int((m["cbc"] != "E  ").sum()) == gold["nbc"]
    assert sorted(set(m["group"].tolist())) == gold["groups"]
    # genbox element order: x fastest; corner 0 of element 1 is the second x lattice value
    assert m["VX"][1, 0, 0] == lat[0][1] and m["VX"][0, 7].tolist() == [lat[0][1], lat[1][1], lat[2][1]]
    # first boundary records of the reference file: (element, face) 1-based, element order
    e, f = np.nonzero(m["cbc"] != "E  ")
    assert [[int(a) + 1, int(b) + 1] for a, b in zip(e[:8], f[:8])] == gold["bc_first"]


def test_boundary_ids_follow_nekrs_face_order(product_lib, kershaw_file):
    p = kershaw_file[0]
    VX, EToV, EToB = R.mesh_from_re2(p, {"O": R.NRSG_BC_DIRICHLET})
    _, _, ref = W.kershaw_box(20, eps=1.0, all_dirichlet=True)
    assert np.array_equal(EToB, ref)


def test_connect_box_numbering(product_lib, kershaw_file):
    VX = kershaw_file[1]
    EToV = R.connect(VX)
    assert np.array_equal(EToV, OR.connect(VX))
    # segments sort by x, then y, then z: z runs fastest
    n = 21
    ix, iy, iz = (np.rint(VX[..., c] / 0.3).astype(np.int64) for c in range(3))
    assert np.array_equal(EToV, 1 + iz + n * (iy + n * ix))


def test_connect_distorted_shuffled_mesh_matches_oracle(product_lib):
    rng = np.random.default_rng(3)
    VX, EToV_box, _ = W.kershaw_box(6, 5, 4, eps=0.3)
    perm = rng.permutation(VX.shape[0])
    VXp = VX[perm]
    ids = R.connect(VXp)
    assert np.array_equal(ids, OR.connect(VXp))
    # same connectivity as the generator's ids, up to renumbering
    ref = EToV_box[perm]
    pairs = set(zip(ids.ravel().tolist(), ref.ravel().tolist()))
    assert len(pairs) == len(set(ids.ravel().tolist())) == len(set(ref.ravel().tolist()))
    # a corner moved by 1e-3 of the edge still joins its neighbours (tol 0.2); by half an edge it does not
    VXq = VXp.copy()
    VXq[0, 0] += 1e-3 * np.abs(VXp[0, 1] - VXp[0, 0]).max()
    assert R.connect(VXq).max() == ids.max()
    VXq[0, 0] = 0.5 * (VXp[0, 0] + VXp[0, 1])
    assert R.connect(VXq).max() == ids.max() + 1


def test_connect_periodic_faces(product_lib, tmp_path):
    n = 4
    xs = np.linspace(0.0, 1.0, n + 1)
    VX, cbc = R.box(n, n, n, xs, xs, xs, ("P", "P", "W", "W", "W", "W"))
    E = VX.shape[0]
    bc = np.zeros((E, 6, 5))
    e = np.arange(E)
    ix, iy, iz = e % n, (e // n) % n, e // (n * n)
    lo, hi = ix == 0, ix == n - 1
    # pre-processor face 3 (r-) of the x- side links to face 1 (r+) of the element at the x+ side
    bc[lo, 3, 0] = (n - 1 + n * (iy + n * iz))[lo] + 1
    bc[lo, 3, 1] = 2
    bc[hi, 1, 0] = (0 + n * (iy + n * iz))[hi] + 1
    bc[hi, 1, 1] = 4
    p = tmp_path / "per.re2"
    R.write_re2(p, VX, cbc, bc)
    m = R.read_re2(p)
    ids = R.connect(m["VX"], 0.2, m["cbc"], m["bc"])
    assert np.array_equal(ids, OR.connect(m["VX"], 0.2, m["cbc"], m["bc"]))
    assert ids.max() == n * (n + 1) * (n + 1)  # the x+ plane of vertices joins the x- plane
    assert np.array_equal(ids[lo][:, [0, 2, 4, 6]], ids[np.flatnonzero(hi)][:, [1, 3, 5, 7]])


@pytest.mark.parametrize("version,byteorder", [(2, ">"), (3, "<"), (4, "<"), (4, ">")])
def test_versions_byte_order_curves_and_sections(product_lib, tmp_path, version, byteorder):
    VX, _, _ = W.kershaw_box(3, 2, 2, eps=0.5)
    VX = VX.copy()
    E = VX.shape[0]
    _, cbc = R.box(3, 2, 2, np.arange(4.0), np.arange(3.0), np.arange(3.0), ("v", "O", "W", "W", "SYM", "W"))
    rng = np.random.default_rng(version)
    bc = rng.standard_normal((E, 6, 5)) * (cbc != "E  ")[..., None]
    cbc2 = np.where(cbc != "E  ", "t  ", "E  ")
    curves = {"elem": np.array([0, 5, 11]), "face": np.array([0, 3, 5]), "params": rng.standard_normal((3, 5)),
              "type": np.array([b"C", b"s", b"m"])}
    group = np.arange(E) % 3
    p = tmp_path / "m.re2"
    R.write_re2(p, VX, cbc, bc, group=group, curves=curves, version=version, nelgv=E - 2, byteorder=byteorder,
                extra_bc=[(cbc2, None)])
    h = R.read_header(p)
    assert (h["version"], h["nelgt"], h["nelgv"], h["ncurve"], h["nbcFields"], h["byteSwapped"]) == \
        (version, E, E - 2, 3, 2, int(byteorder == ">"))
    m0, m1 = R.read_re2(p, 0), R.read_re2(p, 1)
    o = OR.read(p)
    assert np.array_equal(m0["VX"], VX) and np.array_equal(o["VX"], VX)
    assert np.array_equal(m0["group"], group)
    assert np.array_equal(m0["cbc"], cbc) and np.array_equal(m0["bc"], bc)
    assert np.array_equal(m1["cbc"], cbc2) and not m1["bc"].any()
    assert np.array_equal(m0["curves"]["elem"], curves["elem"]) and np.array_equal(m0["curves"]["face"], curves["face"])
    assert np.array_equal(m0["curves"]["params"], curves["params"])
    assert m0["curves"]["type"].tolist() == curves["type"].tolist()


def test_reader_rejects_bad_files(product_lib, tmp_path):
    p = tmp_path / "bad.re2"
    p.write_bytes(b"#v001" + b" " * 100)
    with pytest.raises(G.NrsgError):
        R.read_header(p)
    VX, _, _ = W.kershaw_box(2, eps=0.5)
    _, cbc = R.box(2, 2, 2, np.arange(3.0), np.arange(3.0), np.arange(3.0), ("O",) * 6)
    good = tmp_path / "good.re2"
    R.write_re2(good, VX, cbc)
    data = good.read_bytes()
    (tmp_path / "trunc.re2").write_bytes(data[:-10])
    with pytest.raises(G.NrsgError):
        R.read_re2(tmp_path / "trunc.re2")
    with pytest.raises(G.NrsgError):
        R.read_re2(good, field=1)
    with pytest.raises(G.NrsgError):
        R.read_header(tmp_path / "missing.re2")


def test_solve_setup_from_re2_matches_generator_mesh(product_lib, oracle_mod, tmp_path):
    """The oracle's solve on a mesh read back from .re2 (parCon ids) equals the solve on the generator's mesh
    (other vertex ids, same connectivity): the numbering only names vertices."""
    from oracle import oracle as O

    N, n = 3, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    _, cbc = R.box(n, n, n, np.arange(n + 1.0), np.arange(n + 1.0), np.arange(n + 1.0), ("O",) * 6)
    p = tmp_path / "k.re2"
    R.write_re2(p, VX, cbc)
    VX2, EToV2, EToB2 = R.mesh_from_re2(p, {"O": R.NRSG_BC_DIRICHLET})
    assert np.array_equal(VX2, VX) and np.array_equal(EToB2, EToB) and not np.array_equal(EToV2, EToV)
    opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=500"
    a = O.Elliptic(N, VX, EToV, EToB, opts)
    b = O.Elliptic(N, VX2, EToV2, EToB2, opts)
    rhs = W.box_rhs(N, n, n, n, 4, a.get("ggeo"))
    xa, ia = a.solve(rhs)
    xb, ib = b.solve(rhs)
    assert ia["iterations"] == ib["iterations"]
    assert np.array_equal(xa, xb)


def test_reader_crosses_its_read_chunk(product_lib, tmp_path):
    """The element section is read in chunks of 65536 records: a file with more elements than one chunk reads
    back exactly (corners, groups, boundary codes of the last elements)."""
    nx, ny, nz = 50, 40, 35  # 70000 elements
    xs, ys, zs = np.linspace(0, 1, nx + 1), np.linspace(0, 2, ny + 1) ** 1.5, np.cumsum(np.arange(nz + 1.0))
    VX, cbc = R.box(nx, ny, nz, xs, ys, zs, ("v", "O", "W", "W", "SYM", "W"))
    group = (np.arange(VX.shape[0]) % 7).astype(np.int32)
    p = tmp_path / "big.re2"
    R.write_re2(p, VX, cbc, group=group)
    m = R.read_re2(p)
    assert m["header"]["nelgt"] == 70000
    assert np.array_equal(m["VX"], VX) and np.array_equal(m["group"], group) and np.array_equal(m["cbc"], cbc)
