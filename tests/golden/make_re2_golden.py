"""Generate tests/golden/re2_kershaw.json from the reference's own Kershaw mesh
(nekRS examples/kershaw/kershaw.re2, genbox output for a 20^3 box on
[0, 6]^3 with 'O' on every side).  Run in a checkout that has the reference
tree; the fixture records the file's size and SHA-256, its header, the lattice
coordinates of its corners (exact, as float hex) and its boundary records, so
that tests can rebuild the file byte for byte without the reference present.

    python tests/golden/make_re2_golden.py [path/to/kershaw.re2]
"""
import hashlib
import json
import os
import sys

import numpy as np

SRC = sys.argv[1] if len(sys.argv) > 1 else os.path.join(
    os.environ.get("NEKRS_REFERENCE_ROOT", "/root/reference"), "examples", "kershaw", "kershaw.re2")
b = open(SRC, "rb").read()
hdr = b[:80].decode()
E = int(hdr[5:14])
el = np.frombuffer(b[84:84 + E * 200], "<f8").reshape(E, 25)
off = 84 + E * 200
ncurve = int(np.frombuffer(b[off:off + 8], "<f8")[0])
off += 8 + 64 * ncurve
nbc = int(np.frombuffer(b[off:off + 8], "<f8")[0])
rec = np.frombuffer(b[off + 8:off + 8 + 64 * nbc], dtype=np.dtype([("w", "<f8", 7), ("c", "S8")]))
lat = [np.unique(el[:, 1 + 8 * c:9 + 8 * c]) for c in range(3)]
out = {
    "source": "nekRS examples/kershaw/kershaw.re2",
    "bytes": len(b),
    "sha256": hashlib.sha256(b).hexdigest(),
    "header": hdr,
    "nelgt": E,
    "box": [len(lat[0]) - 1, len(lat[1]) - 1, len(lat[2]) - 1],
    "lattice_hex": [[float(v).hex() for v in a] for a in lat],
    "groups": sorted(set(el[:, 0].tolist())),
    "ncurve": ncurve,
    "nbc": nbc,
    "bc_codes": sorted(set(c.decode() for c in rec["c"])),
    "bc_params_all_zero": bool((rec["w"][:, 2:] == 0).all()),
    "bc_first": [[int(r["w"][0]), int(r["w"][1])] for r in rec[:8]],
}
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "re2_kershaw.json")
json.dump(out, open(dst, "w"), indent=1)
print(dst)
