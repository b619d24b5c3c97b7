"""ctypes front end of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and the cpu-baseline leg of
bench.py, never by the product package.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

D = ctypes.POINTER(ctypes.c_double)
F = ctypes.POINTER(ctypes.c_float)
L = ctypes.POINTER(ctypes.c_longlong)
I = ctypes.POINTER(ctypes.c_int)


def _p(a, t):
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = ctypes.CDLL(path)
        _lib.orc_create.restype = ctypes.c_void_p
        _lib.orc_create.argtypes = [ctypes.c_int, ctypes.c_longlong, D, L, I, ctypes.c_char_p]
        _lib.orc_destroy.argtypes = [ctypes.c_void_p]
        _lib.orc_size.restype = ctypes.c_longlong
        _lib.orc_size.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        _lib.orc_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        _lib.orc_volume.restype = ctypes.c_double
        _lib.orc_volume.argtypes = [ctypes.c_void_p]
        for name in ("orc_ax", "orc_ax_ref", "orc_operator", "orc_precond"):
            getattr(_lib, name).argtypes = [ctypes.c_void_p, D, D]
        _lib.orc_ax_fp32.argtypes = [ctypes.c_void_p, F, F]
        _lib.orc_gs.argtypes = [ctypes.c_void_p, D]
        _lib.orc_mask.argtypes = [ctypes.c_void_p, D]
        _lib.orc_solve.argtypes = [ctypes.c_void_p, D, D, D]
        _lib.orc_box_mesh.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, D, L, I, ctypes.c_int]
        _lib.orc_box_rhs.argtypes = [ctypes.c_int] * 4 + [ctypes.c_ulonglong, D, D]
        _lib.orc_mg_info.restype = ctypes.c_longlong
        _lib.orc_mg_info.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        _lib.orc_mg_level_size.restype = ctypes.c_longlong
        _lib.orc_mg_level_size.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib.orc_mg_schwarz.argtypes = [ctypes.c_void_p, ctypes.c_int, D, D]
        _lib.orc_mg_get.restype = ctypes.c_longlong
        _lib.orc_mg_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p]
        _lib.orc_mg_transfer.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, D, D]
        _lib.orc_hessenberg_rho.restype = ctypes.c_double
        _lib.orc_hessenberg_rho.argtypes = [ctypes.c_int, D]
        _lib.orc_assemble_fem.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int] + \
            [ctypes.c_void_p] * 5
        _lib.orc_global_ids.argtypes = [ctypes.c_int, ctypes.c_longlong, L, L]
        _lib.orc_gll.argtypes = [ctypes.c_int, D, D]
        _lib.orc_wdot.restype = ctypes.c_double
        _lib.orc_wdot.argtypes = [ctypes.c_longlong, ctypes.c_void_p, D, D]
        _lib.orc_update_pcg.restype = ctypes.c_double
        _lib.orc_update_pcg.argtypes = [ctypes.c_longlong, D, D, D, ctypes.c_double, D, D]
        _lib.orc_dmatrix.argtypes = [ctypes.c_int, D]
        _lib.orc_interp.argtypes = [ctypes.c_int, ctypes.c_int, D]
        vp, ci, cd, cl = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
        _lib.orc_assemble_galerkin.argtypes = [vp, vp, cd, cd, ci] + [vp] * 5
        _lib.orc_assemble_semfem.argtypes = [vp, cd] + [vp] * 5
        _lib.orc_block_vgeo.argtypes = [vp, vp]
        _lib.orc_block_ax.argtypes = [vp, ci, ci, ci, cl, vp, vp, cd, cd, vp, vp]
        _lib.orc_block_diag.argtypes = [vp, ci, ci, cl, vp, vp, cd, cd, vp]
        _lib.orc_block_solve.argtypes = [vp, ci, ci, ci, cl, vp, vp, cd, cd, ci, cd, ci, ci, vp, vp, vp, vp]
        _lib.orc_zero_normal.argtypes = [vp, vp, vp, vp]
        _lib.orc_zero_normal.restype = ci
        _lib.orc_apply_zero_normal.argtypes = [vp, vp, vp]
    return _lib


def ref_lib():
    """The reference's own serial kernels (oracle/_ref), or None where absent."""
    global _ref
    if _ref is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libnekref.so")
        if not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
    return _ref


def gll(N):
    z = np.zeros(N + 1)
    w = np.zeros(N + 1)
    lib().orc_gll(N, _p(z, D), _p(w, D))
    return z, w


def wdot(w, a, b):
    """sum_i w_i (a_i b_i) in the device library's reduction order (w None: unweighted)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if w is None:
        return lib().orc_wdot(a.size, None, _p(a, D), _p(b, D))
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib().orc_wdot(a.size, w.ctypes.data_as(ctypes.c_void_p), _p(a, D), _p(b, D))


def update_pcg(w, p, Ap, alpha, x, r):
    """The fused PCG update in place on x and r; returns (r, r)_w."""
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (w, p, Ap)]
    return lib().orc_update_pcg(x.size, _p(arrs[0], D), _p(arrs[1], D), _p(arrs[2], D), alpha, _p(x, D), _p(r, D))


def dmatrix(N):
    Dm = np.zeros((N + 1) * (N + 1))
    lib().orc_dmatrix(N, _p(Dm, D))
    return Dm.reshape(N + 1, N + 1)


def interp(Nin, Nout):
    Im = np.zeros((Nout + 1) * (Nin + 1))
    lib().orc_interp(Nin, Nout, _p(Im, D))
    return Im.reshape(Nout + 1, Nin + 1)


def box_mesh(nx, ny, nz, eps, all_dirichlet=True):
    E = nx * ny * nz
    VX = np.zeros((E, 8, 3))
    EToV = np.zeros((E, 8), dtype=np.int64)
    EToB = np.zeros((E, 6), dtype=np.int32)
    lib().orc_box_mesh(nx, ny, nz, eps, _p(VX, D), _p(EToV, L), _p(EToB, I), 1 if all_dirichlet else 0)
    return VX, EToV, EToB


def global_ids(N, EToV):
    E = EToV.shape[0]
    ids = np.zeros(E * (N + 1) ** 3, dtype=np.int64)
    EToV = np.ascontiguousarray(EToV, dtype=np.int64)
    lib().orc_global_ids(N, E, _p(EToV, L), _p(ids, L))
    return ids


class Elliptic:
    """Oracle solver for one mesh; options use the .par [PRESSURE] keys."""

    def __init__(self, N, VX, EToV, EToB, options=""):
        self.N = N
        self.E = VX.shape[0]
        self.Np = (N + 1) ** 3
        self.Nlocal = self.E * self.Np
        self._VX = np.ascontiguousarray(VX, dtype=np.float64)
        self._EToV = np.ascontiguousarray(EToV, dtype=np.int64)
        self._EToB = np.ascontiguousarray(EToB, dtype=np.int32)
        self.h = lib().orc_create(N, self.E, _p(self._VX, D), _p(self._EToV, L), _p(self._EToB, I),
                                  options.encode())
        if not self.h:
            raise RuntimeError("oracle setup failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def get(self, name):
        n = lib().orc_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        dt = {"ids": np.int64, "maskedIds": np.int64, "gsOff": np.int32, "gsIds": np.int32,
              "maskIds": np.int32}.get(name, np.float64)
        out = np.zeros(n, dtype=dt)
        lib().orc_get(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p))
        return out

    # ---- block (vector) Helmholtz: nf fields at fieldOffset = Nlocal; lam0 / lam1 per node
    # (length Nlocal, or nf*Nlocal with loffset = Nlocal) or None for the scalars l0 / l1
    @staticmethod
    def _lam(a):
        return None if a is None else np.ascontiguousarray(a, dtype=np.float64)

    def block_vgeo(self):
        n = self.get("ggeo").size // 7
        out = np.zeros(12 * n)
        lib().orc_block_vgeo(self.h, out.ctypes.data)
        return out

    def block_ax(self, q, nf=3, stress=False, poisson=False, lam0=None, lam1=None, l0=1.0, l1=0.0, loffset=0):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros_like(q)
        a0, a1 = self._lam(lam0), self._lam(lam1)
        lib().orc_block_ax(self.h, nf, int(stress), int(poisson), loffset, None if a0 is None else a0.ctypes.data,
                           None if a1 is None else a1.ctypes.data, l0, l1, q.ctypes.data, out.ctypes.data)
        return out

    def block_inv_diag(self, nf=3, poisson=False, lam0=None, lam1=None, l0=1.0, l1=0.0, loffset=0):
        n = self.get("invDegree").size
        out = np.zeros(nf * n)
        a0, a1 = self._lam(lam0), self._lam(lam1)
        lib().orc_block_diag(self.h, nf, int(poisson), loffset, None if a0 is None else a0.ctypes.data,
                             None if a1 is None else a1.ctypes.data, l0, l1, out.ctypes.data)
        return out

    def block_solve(self, rhs, nf=3, stress=False, poisson=False, lam0=None, lam1=None, l0=1.0, l1=0.0, loffset=0,
                    jacobi=True, tol=1e-8, relative=True, maxit=1000, x0=None, EToB_fields=None):
        r = np.array(rhs, dtype=np.float64)
        x = np.zeros_like(r) if x0 is None else np.array(x0, dtype=np.float64)
        info = np.zeros(4)
        a0, a1 = self._lam(lam0), self._lam(lam1)
        eb = None if EToB_fields is None else np.ascontiguousarray(EToB_fields, dtype=np.int32)
        lib().orc_block_solve(self.h, nf, int(stress), int(poisson), loffset, None if a0 is None else a0.ctypes.data,
                              None if a1 is None else a1.ctypes.data, l0, l1, int(jacobi), tol, int(relative), maxit,
                              None if eb is None else eb.ctypes.data, r.ctypes.data, x.ctypes.data, info.ctypes.data)
        return x, {"iterations": int(info[0]), "res0": info[1], "res": info[2], "status": int(info[3]), "r": r}

    def zero_normal(self, EToB0):
        """Frames of the zero-normal faces (type 2) of EToB0 [E][6]: sgeo [E][6][Nq^2][9] (n, t1, t2) and the
        mask [3][Nlocal]; None when no face is zero-normal."""
        eb = np.ascontiguousarray(EToB0, dtype=np.int32)
        E = eb.shape[0]
        nl = self.get("invDegree").size
        nq = round((nl // E) ** (1 / 3))
        sgeo = np.zeros((E, 6, nq * nq, 9))
        mask = np.zeros(3 * nl)
        if not lib().orc_zero_normal(self.h, eb.ctypes.data, sgeo.ctypes.data, mask.ctypes.data):
            return None
        return sgeo, mask

    def apply_zero_normal(self, EToB0, U):
        eb = np.ascontiguousarray(EToB0, dtype=np.int32)
        out = np.array(U, dtype=np.float64)
        lib().orc_apply_zero_normal(self.h, eb.ctypes.data, out.ctypes.data)
        return out

    @property
    def volume(self):
        return lib().orc_volume(self.h)

    def ax(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros_like(q)
        lib().orc_ax(self.h, _p(q, D), _p(out, D))
        return out

    def ax_ref(self, q):
        """FP64 Ax in the operation order of the reference's serial kernel."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros_like(q)
        lib().orc_ax_ref(self.h, _p(q, D), _p(out, D))
        return out

    def ax_fp32(self, q):
        q = np.ascontiguousarray(q, dtype=np.float32)
        out = np.zeros_like(q)
        lib().orc_ax_fp32(self.h, _p(q, F), _p(out, F))
        return out

    def operator(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros_like(q)
        lib().orc_operator(self.h, _p(q, D), _p(out, D))
        return out

    def gs(self, q):
        q = np.array(q, dtype=np.float64)
        lib().orc_gs(self.h, _p(q, D))
        return q

    def mask(self, q):
        q = np.array(q, dtype=np.float64)
        lib().orc_mask(self.h, _p(q, D))
        return q

    def precond(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros_like(r)
        lib().orc_precond(self.h, _p(r, D), _p(z, D))
        return z

    def mg_info(self, what):
        n = lib().orc_mg_info(self.h, what.encode(), None)
        out = np.zeros(n)
        if n:
            lib().orc_mg_info(self.h, what.encode(), out.ctypes.data_as(ctypes.c_void_p))
        return out

    def mg_schwarz(self, level, u):
        n = lib().orc_mg_level_size(self.h, level)
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.size == n
        out = np.zeros(n)
        lib().orc_mg_schwarz(self.h, level, _p(u, D), _p(out, D))
        return out

    def mg_get(self, level, name):
        n = lib().orc_mg_get(self.h, level, name.encode(), None)
        out = np.zeros(n)
        if n:
            lib().orc_mg_get(self.h, level, name.encode(), out.ctypes.data_as(ctypes.c_void_p))
        return out

    def mg_transfer(self, level, restrict, v, nout):
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.zeros(nout)
        lib().orc_mg_transfer(self.h, level, 1 if restrict else 0, _p(v, D), _p(out, D))
        return out

    def assemble(self, lambda0=1.0, lambda1=0.0, poisson=True):
        """Assembled operator of this level (CSR: rowPtr, cols, vals), built as the reference's
        FEM coarse-matrix builder does."""
        nrow, nnz = ctypes.c_longlong(0), ctypes.c_longlong(0)
        a = (self.h, float(lambda0), float(lambda1), int(poisson), ctypes.byref(nrow), ctypes.byref(nnz))
        lib().orc_assemble_fem(*a, None, None, None)
        rp = np.zeros(nrow.value + 1, np.int64)
        cols = np.zeros(nnz.value, np.int64)
        vals = np.zeros(nnz.value)
        lib().orc_assemble_fem(*a, rp.ctypes.data_as(ctypes.c_void_p), cols.ctypes.data_as(ctypes.c_void_p),
                               vals.ctypes.data_as(ctypes.c_void_p))
        return rp, cols, vals

    def assemble_semfem(self, lambda0=1.0):
        """SEMFEM operator of this level (linear tetrahedra on its GLL grid), CSR."""
        nrow, nnz = ctypes.c_longlong(0), ctypes.c_longlong(0)
        a = (self.h, float(lambda0), ctypes.byref(nrow), ctypes.byref(nnz))
        lib().orc_assemble_semfem(*a, None, None, None)
        rp = np.zeros(nrow.value + 1, np.int64)
        cols = np.zeros(nnz.value, np.int64)
        vals = np.zeros(nnz.value)
        lib().orc_assemble_semfem(*a, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data)
        return rp, cols, vals

    def assemble_galerkin(self, coarse, lambda0=1.0, lambda1=0.0, poisson=True):
        """Galerkin order-1 operator B^T A B of this (fine) level on the order-1 handle ``coarse`` (same mesh)."""
        nrow, nnz = ctypes.c_longlong(0), ctypes.c_longlong(0)
        a = (self.h, coarse.h, float(lambda0), float(lambda1), int(poisson), ctypes.byref(nrow), ctypes.byref(nnz))
        lib().orc_assemble_galerkin(*a, None, None, None)
        rp = np.zeros(nrow.value + 1, np.int64)
        cols = np.zeros(nnz.value, np.int64)
        vals = np.zeros(nnz.value)
        lib().orc_assemble_galerkin(*a, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data)
        return rp, cols, vals

    def solve(self, rhs, x0=None):
        r = np.array(rhs, dtype=np.float64)
        x = np.zeros_like(r) if x0 is None else np.array(x0, dtype=np.float64)
        info = np.zeros(4)
        lib().orc_solve(self.h, _p(r, D), _p(x, D), _p(info, D))
        return x, {"iterations": int(info[0]), "res0": info[1], "res": info[2], "status": int(info[3]),
                   "history": self.get("history"), "r": r}


def box_rhs(N, nx, ny, nz, seed, ggeo):
    E = nx * ny * nz
    rhs = np.zeros(E * (N + 1) ** 3)
    g = np.ascontiguousarray(ggeo, dtype=np.float64)
    lib().orc_box_rhs(N, nx, ny, nz, seed, _p(g, D), _p(rhs, D))
    return rhs


def hessenberg_rho(n, Hcol):
    Hcol = np.ascontiguousarray(Hcol, dtype=np.float64)
    return lib().orc_hessenberg_rho(n, _p(Hcol, D))
