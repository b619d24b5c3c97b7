"""nekrs_gb300 — GB300-native pressure/Helmholtz elliptic solve.

Python front end of the C ABI declared in include/nekrs_gb300.h.  The compute
path is the in-tree CUDA library nekrs_gb300/_lib/libnekrs_gb300.so (built for
sm_103a by nekrs_gb300._build); there is no CPU fallback: if the library or a
CUDA device is missing, every call raises.

Device buffers are passed as objects exposing ``data_ptr()`` (e.g. torch CUDA
tensors) or as raw integer device addresses.
"""
import ctypes
import os

import numpy as np

from . import workloads  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnekrs_gb300.so")

NRSG_OK = 0
STATUS = {0: "OK", 1: "MAXIT", 2: "BREAKDOWN", 3: "NAN", 4: "OOM", 5: "BAD_CONFIG", 6: "CUDA", 7: "NO_DEVICE",
          8: "INVALID"}

_lib = None
vp = ctypes.c_void_p
LL = ctypes.c_longlong


class NrsgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nekrs_gb300 error {code} ({STATUS.get(code, '?')}): {msg}")
        self.code = code


class MeshDesc(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("Nelements", LL), ("h_VX", vp), ("h_EToV", vp), ("h_EToB", vp),
                ("h_ggeo", vp)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("status", ctypes.c_int), ("res0", ctypes.c_double),
                ("res", ctypes.c_double), ("solve_ms", ctypes.c_double)]

    def as_dict(self):
        return {"iterations": self.iterations, "status": self.status, "res0": self.res0, "res": self.res,
                "solve_ms": self.solve_ms}


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"nekrs_gb300 CUDA library not built ({LIB_PATH}); run nekrs_gb300._build.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.nrsg_last_error.restype = ctypes.c_char_p
        L.nrsg_kernel_launches.restype = LL
        L.nrsg_host_hessenberg_rho.restype = ctypes.c_double
        L.nrsg_host_hessenberg_rho.argtypes = [ctypes.c_int, vp]
        L.nrsg_host_setup_maps.argtypes = [ctypes.c_int, LL] + [vp] * 10
        L.nrsg_host_assemble_operator.argtypes = ([ctypes.c_int, LL, vp, vp, vp, ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_int] + [vp] * 6)
        L.nrsg_host_assemble_galerkin.argtypes = ([ctypes.c_int, LL, vp, vp, vp, ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_int] + [vp] * 6)
        L.nrsg_host_assemble_semfem.argtypes = [ctypes.c_int, LL, vp, vp, vp, ctypes.c_double] + [vp] * 6
        L.nrsg_amg_create.argtypes = [LL, vp, vp, vp, ctypes.POINTER(vp)]
        L.nrsg_amg_destroy.argtypes = [vp]
        L.nrsg_amg_num_levels.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        L.nrsg_amg_level_matrix.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(LL), ctypes.POINTER(LL),
                                            ctypes.POINTER(LL), vp, vp, vp, ctypes.POINTER(ctypes.c_double)]
        L.nrsg_amg_vcycle.argtypes = [vp, vp, vp, vp]
        L.nrsg_elliptic_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.c_char_p, ctypes.POINTER(vp)]
        L.nrsg_elliptic_destroy.argtypes = [vp]
        L.nrsg_elliptic_set_stream.argtypes = [vp, vp]
        L.nrsg_elliptic_solve.argtypes = [vp, vp, vp, ctypes.POINTER(SolveInfo)]
        L.nrsg_elliptic_solve_host.argtypes = [vp, vp, vp, ctypes.POINTER(SolveInfo)]
        L.nrsg_elliptic_solve_begin.argtypes = [vp, vp, vp]
        L.nrsg_elliptic_set_tolerance.argtypes = [vp, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.nrsg_elliptic_set_coefficients.argtypes = [vp, vp, vp, LL]
        L.nrsg_elliptic_set_field_bcs.argtypes = [vp, vp]
        L.nrsg_elliptic_solve_advance.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(SolveInfo)]
        L.nrsg_server_create.argtypes = [LL, ctypes.POINTER(vp)]
        L.nrsg_server_destroy.argtypes = [vp]
        L.nrsg_server_submit.argtypes = [vp, vp, vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, LL,
                                         ctypes.POINTER(LL)]
        L.nrsg_server_step.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.nrsg_server_poll.argtypes = [vp, ctypes.POINTER(LL), ctypes.POINTER(SolveInfo), ctypes.POINTER(ctypes.c_int)]
        L.nrsg_elliptic_solve_batch.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                                ctypes.POINTER(vp), ctypes.POINTER(SolveInfo)]
        for f in ("nrsg_elliptic_operator", "nrsg_elliptic_ax", "nrsg_elliptic_precondition"):
            getattr(L, f).argtypes = [vp, vp, vp]
        L.nrsg_elliptic_gs.argtypes = [vp, vp]
        L.nrsg_elliptic_mask.argtypes = [vp, vp]
        L.nrsg_elliptic_get.argtypes = [vp, ctypes.c_char_p, vp, ctypes.POINTER(LL)]
        L.nrsg_elliptic_mg_smoother.argtypes = [vp, ctypes.c_int, vp, vp]
        L.nrsg_elliptic_mg_fdm.argtypes = [vp, ctypes.c_int, vp, vp]
        L.nrsg_elliptic_mg_level_size.restype = LL
        L.nrsg_elliptic_mg_level_size.argtypes = [vp, ctypes.c_int]
        d, f, i = ctypes.c_double, ctypes.c_float, ctypes.c_int
        L.nrsg_ax_stored_f64.argtypes = [i, LL, vp, vp, d, d, i, vp, vp, vp]
        L.nrsg_ax_stored_f32.argtypes = [i, LL, vp, vp, f, f, i, vp, vp, vp]
        L.nrsg_ax_pipe_f32.argtypes = [i, LL, vp, vp, f, f, i, vp, vp, vp]
        L.nrsg_ax_const_f32.argtypes = [i, LL, vp, vp, f, f, i, vp, vp, vp]
        L.nrsg_ax_const_prefetch_f32.argtypes = [i, LL, vp, vp, f, f, i, vp, vp, vp]
        L.nrsg_ax_trilinear_f64.argtypes = [i, LL, vp, vp, vp, vp, d, d, i, vp, vp, vp]
        L.nrsg_ax_trilinear_f32.argtypes = [i, LL, vp, vp, vp, vp, f, f, i, vp, vp, vp]
        L.nrsg_ax_fp32x2.argtypes = [i, LL, vp, vp, d, d, i, vp, vp, vp]
        L.nrsg_split_pairs.argtypes = [LL, vp, vp, vp]
        L.nrsg_gs_add_f64.argtypes = [LL, vp, vp, vp, vp]
        L.nrsg_gs_add_f32.argtypes = [LL, vp, vp, vp, vp]
        L.nrsg_mask_f64.argtypes = [LL, vp, vp, vp]
        L.nrsg_update_pcg_f64.argtypes = [LL, vp, vp, vp, d, vp, vp, vp, vp]
        L.nrsg_weighted_inner_prod_f64.argtypes = [LL, vp, vp, vp, vp, vp]
        L.nrsg_geometric_factors_f64.argtypes = [i, LL, vp, vp, vp]
        _lib = L
    return _lib


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError("expected a device buffer with data_ptr() or an int address")


def check(code):
    if code != NRSG_OK:
        raise NrsgError(code, lib().nrsg_last_error().decode(errors="replace"))
    return code


_DTYPES = {"ids": np.int64, "maskedIds": np.int64, "gsOff": np.int32, "gsIds": np.int32, "maskIds": np.int32}


class Elliptic:
    """GB300 counterpart of one ``elliptic_t`` (ellipticSolveSetup + ellipticSolve).

    ``options`` uses the .par [PRESSURE]-section keys, one ``key = value`` per
    line or ';'-separated.
    """

    def __init__(self, N, VX, EToV, EToB, options="", ggeo=None):
        self.N = int(N)
        self._VX = np.ascontiguousarray(VX, dtype=np.float64)
        self._EToV = np.ascontiguousarray(EToV, dtype=np.int64)
        self._EToB = np.ascontiguousarray(EToB, dtype=np.int32)
        self.E = self._VX.shape[0]
        self.Np = (self.N + 1) ** 3
        self.Nlocal = self.E * self.Np
        self._ggeo = None if ggeo is None else np.ascontiguousarray(ggeo, dtype=np.float64)
        desc = MeshDesc(self.N, self.E, self._VX.ctypes.data, self._EToV.ctypes.data, self._EToB.ctypes.data,
                        None if self._ggeo is None else self._ggeo.ctypes.data)
        h = vp()
        check(lib().nrsg_elliptic_create(ctypes.byref(desc), options.encode(), ctypes.byref(h)))
        self.h = h
        self._stream = None  # None: the library's own stream

    def close(self):
        if getattr(self, "h", None):
            lib().nrsg_elliptic_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        check(lib().nrsg_elliptic_set_stream(self.h, stream_handle))
        self._stream = stream_handle

    def _order_with(self, *bufs):
        """Given torch CUDA tensors, run the library on the caller's current torch stream, so that the
        caller's earlier writes to the buffers and later reads of them are ordered with its kernels (the
        library's own stream is non-blocking and would not wait for them)."""
        for b in bufs:
            if getattr(b, "is_cuda", False):
                import torch

                s = torch.cuda.current_stream(b.device).cuda_stream
                if s != self._stream:
                    self.set_stream(s)
                return

    def solve(self, r, x):
        """ellipticSolve(elliptic, r, x) on device E-vectors; r becomes the residual."""
        self._order_with(r, x)
        info = SolveInfo()
        code = lib().nrsg_elliptic_solve(self.h, _ptr(r), _ptr(x), ctypes.byref(info))
        if code not in (NRSG_OK, 1):
            check(code)
        return info.as_dict()

    def _own_stream(self):
        """A stream of this handle alone (batched and resumable solves run handles concurrently); waits for
        the caller's current torch stream so that buffers it wrote are in place."""
        import torch

        torch.cuda.current_stream().synchronize()
        if getattr(self, "_batch_stream", None) is None:
            self._batch_stream = torch.cuda.Stream()
        s = self._batch_stream.cuda_stream
        if s != self._stream:
            self.set_stream(s)

    def set_coefficients(self, lambda0, lambda1=None, loffset=0):
        """Per-node coefficient fields (device buffers of E*Np, or nFields*E*Np with loffset = E*Np)."""
        self._order_with(lambda0, lambda1)
        check(lib().nrsg_elliptic_set_coefficients(self.h, _ptr(lambda0), _ptr(lambda1), loffset))

    def set_field_bcs(self, EToB_fields):
        """Boundary types per field of a block solve: int array [nFields, E, 6] (nekRS face order)."""
        b = np.ascontiguousarray(EToB_fields, dtype=np.int32)
        check(lib().nrsg_elliptic_set_field_bcs(self.h, b.ctypes.data))

    def set_tolerance(self, tol, relative=True, max_iterations=400):
        check(lib().nrsg_elliptic_set_tolerance(self.h, float(tol), int(relative), int(max_iterations)))

    def solve_begin(self, r, x):
        """Queue a resumable solve (see solve_advance); r and x are device E-vectors."""
        self._own_stream()
        check(lib().nrsg_elliptic_solve_begin(self.h, _ptr(r), _ptr(x)))

    def solve_advance(self):
        """Advance the resumable solve without waiting on the device: None while running, else the info dict."""
        done = ctypes.c_int(0)
        info = SolveInfo()
        code = lib().nrsg_elliptic_solve_advance(self.h, ctypes.byref(done), ctypes.byref(info))
        if not done.value:
            return None
        if code not in (NRSG_OK, 1):
            check(code)
        return info.as_dict()

    def solve_host(self, r, x):
        """Same solve on host numpy arrays (copied in and out)."""
        assert r.dtype == np.float64 and x.dtype == np.float64 and r.flags.c_contiguous and x.flags.c_contiguous
        info = SolveInfo()
        code = lib().nrsg_elliptic_solve_host(self.h, r.ctypes.data, x.ctypes.data, ctypes.byref(info))
        if code not in (NRSG_OK, 1):
            check(code)
        return info.as_dict()

    def solve_host_ptr(self, r_ptr, x_ptr):
        """Host solve on raw host addresses (e.g. pinned torch CPU tensors)."""
        info = SolveInfo()
        code = lib().nrsg_elliptic_solve_host(self.h, _ptr(r_ptr), _ptr(x_ptr), ctypes.byref(info))
        if code not in (NRSG_OK, 1):
            check(code)
        return info.as_dict()

    def operator(self, q, Aq):
        self._order_with(q, Aq)
        check(lib().nrsg_elliptic_operator(self.h, _ptr(q), _ptr(Aq)))

    def ax(self, q, Aq):
        self._order_with(q, Aq)
        check(lib().nrsg_elliptic_ax(self.h, _ptr(q), _ptr(Aq)))

    def gs(self, q):
        self._order_with(q)
        check(lib().nrsg_elliptic_gs(self.h, _ptr(q)))

    def mask(self, q):
        self._order_with(q)
        check(lib().nrsg_elliptic_mask(self.h, _ptr(q)))

    def precondition(self, r, z):
        self._order_with(r, z)
        check(lib().nrsg_elliptic_precondition(self.h, _ptr(r), _ptr(z)))

    def mg_smoother(self, level, u, Su):
        self._order_with(u, Su)
        check(lib().nrsg_elliptic_mg_smoother(self.h, level, _ptr(u), _ptr(Su)))

    def mg_fdm(self, level, u, Su):
        """One fused FDM launch of a level on buffers of the multigrid precision (asynchronous)."""
        self._order_with(u, Su)
        check(lib().nrsg_elliptic_mg_fdm(self.h, level, _ptr(u), _ptr(Su)))

    def mg_level_size(self, level):
        return lib().nrsg_elliptic_mg_level_size(self.h, level)

    def get(self, name):
        n = LL(0)
        check(lib().nrsg_elliptic_get(self.h, name.encode(), None, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=_DTYPES.get(name, np.float64))
        if n.value:
            check(lib().nrsg_elliptic_get(self.h, name.encode(), out.ctypes.data, ctypes.byref(n)))
        return out


def kernel_launches():
    """Kernels launched by the library so far in this process."""
    return lib().nrsg_kernel_launches()


def host_hessenberg_rho(n, Hcol):
    """Spectral radius of a column-major upper-Hessenberg matrix (host code of the library)."""
    H = np.ascontiguousarray(Hcol, dtype=np.float64)
    return lib().nrsg_host_hessenberg_rho(n, H.ctypes.data)


def host_setup_maps(N, EToV, EToB):
    """Numbering, mask and masked gather maps computed by the library on the host."""
    EToV = np.ascontiguousarray(EToV, dtype=np.int64)
    EToB = np.ascontiguousarray(EToB, dtype=np.int32)
    E = EToV.shape[0]
    n = E * (N + 1) ** 3
    ids = np.zeros(n, np.int64)
    masked = np.zeros(n, np.int64)
    inv = np.zeros(n)
    mask = np.zeros(n, np.int32)
    off = np.zeros(n + 1, np.int32)
    gids = np.zeros(n, np.int32)
    nm, ng = LL(0), LL(0)
    check(lib().nrsg_host_setup_maps(N, E, EToV.ctypes.data, EToB.ctypes.data, ids.ctypes.data, masked.ctypes.data,
                                     inv.ctypes.data, mask.ctypes.data, ctypes.byref(nm), off.ctypes.data,
                                     ctypes.byref(ng), gids.ctypes.data))
    off = off[: ng.value + 1]
    return {"ids": ids, "maskedIds": masked, "invDegree": inv, "maskIds": mask[: nm.value], "gsOff": off,
            "gsIds": gids[: off[-1]]}


class Amg:
    """Algebraic multigrid of an assembled SPD operator (the coarse solve of coarseSolver = amg): the hierarchy
    is built on the host at construction (CSR, 0-based), vcycle runs one V-cycle on the device."""

    def __init__(self, rowPtr, cols, vals):
        rp = np.ascontiguousarray(rowPtr, dtype=np.int64)
        ci = np.ascontiguousarray(cols, dtype=np.int64)
        va = np.ascontiguousarray(vals, dtype=np.float64)
        self.n = len(rp) - 1
        h = ctypes.c_void_p()
        check(lib().nrsg_amg_create(self.n, rp.ctypes.data, ci.ctypes.data, va.ctypes.data, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            lib().nrsg_amg_destroy(self.h)
            self.h = None

    @property
    def num_levels(self):
        n = ctypes.c_int()
        check(lib().nrsg_amg_num_levels(self.h, ctypes.byref(n)))
        return n.value

    def level_matrix(self, level, which=0):
        """(rowPtr, cols, vals, shape, lmax) of level `level`'s operator (which=0) or interpolation (which=1)."""
        nr, nc, nz = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        lm = ctypes.c_double()
        check(lib().nrsg_amg_level_matrix(self.h, level, which, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(nz),
                                          None, None, None, ctypes.byref(lm)))
        rp = np.zeros(nr.value + 1, dtype=np.int64)
        ci = np.zeros(nz.value, dtype=np.int32)
        va = np.zeros(nz.value)
        check(lib().nrsg_amg_level_matrix(self.h, level, which, None, None, None, rp.ctypes.data, ci.ctypes.data,
                                          va.ctypes.data, None))
        return rp, ci, va, (nr.value, nc.value), lm.value

    def vcycle(self, b, x, stream=None):
        """One V-cycle from x = 0 on device FP64 vectors (torch tensors or pointers)."""
        check(lib().nrsg_amg_vcycle(self.h, _ptr(b), _ptr(x), stream))


def host_assemble_operator(N, EToV, EToB, ggeo, lambda0=1.0, lambda1=0.0, poisson=True):
    """Assembled level operator on the unmasked unique nodes (CSR) computed by the library on the host:
    (rowPtr, cols, vals, rowOfNode)."""
    EToV = np.ascontiguousarray(EToV, dtype=np.int64)
    EToB = np.ascontiguousarray(EToB, dtype=np.int32)
    ggeo = np.ascontiguousarray(ggeo, dtype=np.float64)
    E = EToV.shape[0]
    nrow, nnz = LL(0), LL(0)
    args = (N, E, EToV.ctypes.data, EToB.ctypes.data, ggeo.ctypes.data, float(lambda0), float(lambda1), int(poisson))
    check(lib().nrsg_host_assemble_operator(*args, ctypes.byref(nrow), ctypes.byref(nnz), None, None, None, None))
    rp = np.zeros(nrow.value + 1, np.int64)
    cols = np.zeros(nnz.value, np.int64)
    vals = np.zeros(nnz.value)
    rown = np.zeros(E * (N + 1) ** 3, np.int64)
    check(lib().nrsg_host_assemble_operator(*args, ctypes.byref(nrow), ctypes.byref(nnz), rp.ctypes.data,
                                            cols.ctypes.data, vals.ctypes.data, rown.ctypes.data))
    return rp, cols, vals, rown


def host_assemble_galerkin(Nf, EToV, EToB, ggeo_fine, lambda0=1.0, lambda1=0.0, poisson=True):
    """Galerkin order-1 coarse operator B^T A_f B (host code of the library): (rowPtr, cols, vals, rowOfNode)."""
    EToV = np.ascontiguousarray(EToV, dtype=np.int64)
    EToB = np.ascontiguousarray(EToB, dtype=np.int32)
    g = np.ascontiguousarray(ggeo_fine, dtype=np.float64)
    E = EToV.shape[0]
    nrow, nnz = LL(0), LL(0)
    a = (Nf, E, EToV.ctypes.data, EToB.ctypes.data, g.ctypes.data, float(lambda0), float(lambda1), int(poisson),
         ctypes.byref(nrow), ctypes.byref(nnz))
    check(lib().nrsg_host_assemble_galerkin(*a, None, None, None, None))
    rp = np.zeros(nrow.value + 1, np.int64)
    cols = np.zeros(nnz.value, np.int64)
    vals = np.zeros(nnz.value)
    ron = np.zeros(E * 8, np.int64)
    check(lib().nrsg_host_assemble_galerkin(*a, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data, ron.ctypes.data))
    return rp, cols, vals, ron


def host_assemble_semfem(N, VX, EToV, EToB, lambda0=1.0):
    """SEMFEM operator (linear tetrahedra on the order-N GLL grid; host code of the library):
    (rowPtr, cols, vals, rowOfNode)."""
    VX = np.ascontiguousarray(VX, dtype=np.float64)
    EToV = np.ascontiguousarray(EToV, dtype=np.int64)
    EToB = np.ascontiguousarray(EToB, dtype=np.int32)
    E = EToV.shape[0]
    nrow, nnz = LL(0), LL(0)
    a = (N, E, VX.ctypes.data, EToV.ctypes.data, EToB.ctypes.data, float(lambda0), ctypes.byref(nrow), ctypes.byref(nnz))
    check(lib().nrsg_host_assemble_semfem(*a, None, None, None, None))
    rp = np.zeros(nrow.value + 1, np.int64)
    cols = np.zeros(nnz.value, np.int64)
    vals = np.zeros(nnz.value)
    ron = np.zeros(E * (N + 1) ** 3, np.int64)
    check(lib().nrsg_host_assemble_semfem(*a, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data, ron.ctypes.data))
    return rp, cols, vals, ron


def solve_batch(solvers, rs, xs):
    """Independent solves on distinct handles, stepped together one Krylov iteration at a time
    (nrsg_elliptic_solve_batch); returns the list of info dicts."""
    n = len(solvers)
    for el in solvers:
        el._own_stream()
    H = (vp * n)(*[el.h for el in solvers])
    R = (vp * n)(*[_ptr(r) for r in rs])
    X = (vp * n)(*[_ptr(x) for x in xs])
    infos = (SolveInfo * n)()
    code = lib().nrsg_elliptic_solve_batch(n, H, R, X, infos)
    if code not in (NRSG_OK, 1):
        check(code)
    return [infos[k].as_dict() for k in range(n)]


# ---- kernel-level entry points ---------------------------------------------
def ax_stored_f64(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_stored_f64(N, E, _ptr(ggeo), _ptr(D), lambda0, lambda1, int(poisson), _ptr(q), _ptr(Aq), stream))


def ax_stored_f32(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_stored_f32(N, E, _ptr(ggeo), _ptr(D), lambda0, lambda1, int(poisson), _ptr(q), _ptr(Aq), stream))


def ax_pipe_f32(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_pipe_f32(N, E, _ptr(ggeo), _ptr(D), lambda0, lambda1, int(poisson), _ptr(q), _ptr(Aq), stream))


def ax_const_f32(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_const_f32(N, E, _ptr(ggeo), _ptr(D), lambda0, lambda1, int(poisson), _ptr(q), _ptr(Aq), stream))


def ax_const_prefetch_f32(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_const_prefetch_f32(N, E, _ptr(ggeo), _ptr(D), lambda0, lambda1, int(poisson), _ptr(q),
                                           _ptr(Aq), stream))


def ax_trilinear_f64(N, E, VX, z, w, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_trilinear_f64(N, E, _ptr(VX), _ptr(z), _ptr(w), _ptr(D), lambda0, lambda1, int(poisson),
                                      _ptr(q), _ptr(Aq), stream))


def ax_trilinear_f32(N, E, VX, z, w, D, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_trilinear_f32(N, E, _ptr(VX), _ptr(z), _ptr(w), _ptr(D), lambda0, lambda1, int(poisson),
                                      _ptr(q), _ptr(Aq), stream))


def ax_fp32x2(N, E, ggeo_pairs, D_pairs, lambda0, lambda1, poisson, q, Aq, stream=0):
    check(lib().nrsg_ax_fp32x2(N, E, _ptr(ggeo_pairs), _ptr(D_pairs), lambda0, lambda1, int(poisson), _ptr(q),
                               _ptr(Aq), stream))


def split_pairs(n, x, pairs, stream=0):
    check(lib().nrsg_split_pairs(n, _ptr(x), _ptr(pairs), stream))


def gs_add_f64(ngroups, off, ids, q, stream=0):
    check(lib().nrsg_gs_add_f64(ngroups, _ptr(off), _ptr(ids), _ptr(q), stream))


def mask_f64(n, ids, q, stream=0):
    check(lib().nrsg_mask_f64(n, _ptr(ids), _ptr(q), stream))


def update_pcg_f64(n, w, p, Ap, alpha, x, r, rdotr, stream=0):
    check(lib().nrsg_update_pcg_f64(n, _ptr(w), _ptr(p), _ptr(Ap), alpha, _ptr(x), _ptr(r), _ptr(rdotr), stream))


def weighted_inner_prod_f64(n, w, a, b, out, stream=0):
    check(lib().nrsg_weighted_inner_prod_f64(n, _ptr(w), _ptr(a), _ptr(b), _ptr(out), stream))


def geometric_factors_f64(N, E, VX, ggeo, stream=0):
    check(lib().nrsg_geometric_factors_f64(N, E, _ptr(VX), _ptr(ggeo), stream))


class Server:
    """Request scheduler over resident operator handles (nrsg_server_*): submit() queues a solve, step()
    admits requests by arrival order and HBM budget and advances every request in flight by at most one
    Krylov iteration, poll() returns finished requests as (request id, info dict)."""

    def __init__(self, hbm_budget_bytes):
        h = ctypes.c_void_p()
        check(lib().nrsg_server_create(int(hbm_budget_bytes), ctypes.byref(h)))
        self.h = h.value
        self._keep = {}

    def __del__(self):
        if getattr(self, "h", None):
            lib().nrsg_server_destroy(self.h)
            self.h = None

    def submit(self, el, r, x, tol, relative=True, max_iterations=400, footprint_bytes=None):
        """Queue a solve of handle `el` on device E-vectors r (overwritten) and x (initial guess / solution)."""
        el._own_stream()  # the handle's own stream; buffers the caller's torch stream wrote are in place
        if footprint_bytes is None:
            footprint_bytes = int(el.get("deviceBytes")[0])
        rid = LL(0)
        check(lib().nrsg_server_submit(self.h, el.h, _ptr(r), _ptr(x), float(tol), int(relative),
                                       int(max_iterations), int(footprint_bytes), ctypes.byref(rid)))
        self._keep[rid.value] = (el, r, x)
        return rid.value

    def step(self):
        """One scheduling step; returns (in flight, queued)."""
        a, q = ctypes.c_int(0), ctypes.c_int(0)
        check(lib().nrsg_server_step(self.h, ctypes.byref(a), ctypes.byref(q)))
        return a.value, q.value

    def poll(self):
        """All finished requests so far: a list of (request id, info dict)."""
        out = []
        while True:
            rid, info, got = LL(0), SolveInfo(), ctypes.c_int(0)
            code = lib().nrsg_server_poll(self.h, ctypes.byref(rid), ctypes.byref(info), ctypes.byref(got))
            if not got.value:
                return out
            self._keep.pop(rid.value, None)
            if code != NRSG_OK:
                raise NrsgError(code, lib().nrsg_last_error().decode(errors="replace"))
            out.append((rid.value, info.as_dict()))
