"""Generate the golden fixtures in tests/golden from the reference's own
serial kernels (oracle/_ref/libnekref.so, built by oracle/build_ref.py from
the reference tree).  Run here, where the reference is mounted; the fixtures
travel with the repository so the GPU host can check against them.

    python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def ref_ax(ref, N, E, ggeo, D, q, poisson, lam0=1.0, lam1=0.0, prec="d"):
    Nq = N + 1
    DT = np.ascontiguousarray(D.reshape(Nq, Nq).T).ravel()
    f = getattr(ref, f"ref_ax_{prec}_{'p' if poisson else 'h'}_N{N}")
    ty = np.float64 if prec == "d" else np.float32
    q = np.ascontiguousarray(q, dtype=ty)
    out = np.zeros_like(q)
    l0 = np.array([lam0], dtype=ty)
    l1 = np.array([lam1], dtype=ty)
    el = np.arange(E, dtype=np.int32)
    cE, off, lo = ctypes.c_int(E), ctypes.c_int(E * Nq ** 3), ctypes.c_int(0)
    f(ctypes.byref(cE), ctypes.byref(off), ctypes.byref(lo), P(el), P(np.ascontiguousarray(ggeo, dtype=ty)),
      P(np.ascontiguousarray(D, dtype=ty)), P(np.ascontiguousarray(DT, dtype=ty)), P(l0), P(l1), P(q), P(out))
    return out


def main():
    build_ref.build()
    ref = O.ref_lib()
    assert ref is not None, "reference kernels not built"
    cases = {}
    rng = np.random.default_rng(20261204)
    for (N, n, eps) in [(3, 2, 0.3), (7, 2, 0.3)]:
        VX, EToV, EToB = O.box_mesh(n, 1, 1, eps)
        el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
        E = VX.shape[0]
        g = el.get("ggeo")
        D = el.get("D")
        q = rng.uniform(-1, 1, E * (N + 1) ** 3)
        tag = f"N{N}"
        cases[f"{tag}_VX"] = VX
        cases[f"{tag}_ggeo"] = g
        cases[f"{tag}_D"] = D
        cases[f"{tag}_q"] = q
        cases[f"{tag}_Aq_poisson"] = ref_ax(ref, N, E, g, D, q, True)
        cases[f"{tag}_Aq_helmholtz"] = ref_ax(ref, N, E, g, D, q, False, 1.3, 0.7)
        cases[f"{tag}_Aq_poisson_f32"] = ref_ax(ref, N, E, g, D, q, True, prec="f")
    np.savez_compressed(os.path.join(OUT, "ref_kernels.npz"), **cases)
    print("wrote", os.path.join(OUT, "ref_kernels.npz"))


if __name__ == "__main__":
    main()
