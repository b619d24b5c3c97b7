"""CPU oracle checks: pinned against the reference's own serial kernels
(oracle/_ref, when built here) and against the committed golden fixtures."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz")


def test_gll_and_derivative(oracle_mod):
    for N in range(1, 10):
        z, w = O.gll(N)
        # exactness of GLL quadrature for degree 2N-1
        for p in range(2 * N):
            exact = (1 - (-1) ** (p + 1)) / (p + 1)
            assert abs(np.dot(w, z ** p) - exact) < 1e-13
        D = O.dmatrix(N)
        for p in range(N + 1):
            assert np.allclose(D @ z ** p, p * z ** max(p - 1, 0) if p else 0 * z, atol=1e-12)


def test_interp_reproduces_polynomials(oracle_mod):
    for (Nf, Nc) in [(7, 3), (3, 1), (9, 5), (5, 3)]:
        Im = O.interp(Nc, Nf)  # coarse -> fine
        zc, _ = O.gll(Nc)
        zf, _ = O.gll(Nf)
        for p in range(Nc + 1):
            assert np.allclose(Im @ zc ** p, zf ** p, atol=1e-13)


@pytest.mark.parametrize("N,n", [(1, 3), (2, 3), (4, 2), (7, 2), (9, 2)])
def test_global_ids_match_coordinates(oracle_mod, N, n):
    VX, EToV, EToB = O.box_mesh(n, n, n, 0.3)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    ids = el.get("ids")
    x, y, z = el.get("x"), el.get("y"), el.get("z")
    key = np.round(np.stack([x, y, z], 1) * 1e9).astype(np.int64)
    nz = ids != 0
    # same id <=> same physical node; interiors (id 0) are exactly the element interiors
    _, inv_p = np.unique(key[nz], axis=0, return_inverse=True)
    _, inv_i = np.unique(ids[nz], return_inverse=True)
    assert np.array_equal(inv_p.ravel(), inv_i.ravel()[np.argsort(np.argsort(inv_i.ravel()))]) or \
        len(np.unique(np.stack([inv_p.ravel(), inv_i.ravel()], 1), axis=0)) == len(np.unique(inv_i))
    assert (ids == 0).sum() == n ** 3 * max(N - 1, 0) ** 3
    # unique non-interior nodes of the box lattice
    L = n * N + 1
    assert ids.max() == L ** 3 - n ** 3 * max(N - 1, 0) ** 3


def test_gather_sanity(oracle_mod):
    # ogs sum test of meshParallelGatherScatterSetup.cpp:136-165 on the unmasked maps
    VX, EToV, EToB = O.box_mesh(3, 2, 2, 0.3)
    N = 5
    el = O.Elliptic(N, VX, EToV, np.zeros_like(EToB), "preconditioner=jacobi")
    one = np.ones(el.Nlocal)
    s = el.gs(one) * el.get("invDegree")
    assert abs(s.sum() - el.Nlocal) / el.Nlocal < 1e-15


def test_oracle_ax_matches_golden(oracle_mod):
    g = np.load(GOLD)
    for N in (3, 7):
        VX = g[f"N{N}_VX"]
        E = VX.shape[0]
        n = E
        _, EToV, EToB = O.box_mesh(n, 1, 1, 0.3)
        el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
        assert np.allclose(el.get("ggeo"), g[f"N{N}_ggeo"], rtol=1e-13, atol=1e-13)
        q = g[f"N{N}_q"]
        ref = g[f"N{N}_Aq_poisson"]
        assert np.max(np.abs(el.ax(q) - ref)) <= 1e-13 * np.max(np.abs(ref))
        el2 = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi;poisson=0;lambda0=1.3;lambda1=0.7")
        refh = g[f"N{N}_Aq_helmholtz"]
        assert np.max(np.abs(el2.ax(q) - refh)) <= 1e-13 * np.max(np.abs(refh))
        ref32 = g[f"N{N}_Aq_poisson_f32"]
        assert np.max(np.abs(el.ax_fp32(q) - ref32)) <= 1e-6 * np.max(np.abs(ref32))


@pytest.mark.skipif(O.ref_lib() is None, reason="reference kernels (oracle/_ref) not built on this host")
@pytest.mark.parametrize("N", [1, 2, 3, 5, 7, 9])
def test_oracle_ax_bitexact_vs_reference(oracle_mod, N):
    import ctypes

    from tests.golden.make_golden import ref_ax

    VX, EToV, EToB = O.box_mesh(2, 2, 1, 0.5)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    rng = np.random.default_rng(N)
    q = rng.uniform(-1, 1, el.Nlocal)
    ref = ref_ax(O.ref_lib(), N, el.E, el.get("ggeo"), el.get("D"), q, True)
    assert np.array_equal(el.ax_ref(q), ref)
    # the device-order operator (fused multiply-adds) agrees to the reference's own
    # acceptance bar for Ax variants: 400 eps relative (benchmarkAx.cpp:295)
    assert np.max(np.abs(el.ax(q) - ref)) <= 400 * np.finfo(np.float64).eps * np.max(np.abs(ref))


@pytest.mark.parametrize("solver", ["pcg", "pfcg", "pgmres", "pfgmres"])
def test_oracle_krylov_converges(oracle_mod, solver):
    VX, EToV, EToB = O.box_mesh(3, 3, 3, 0.3)
    N = 4
    el = O.Elliptic(N, VX, EToV, EToB, f"preconditioner=jacobi;solver={solver};residualTol=1e-8+relative;maxIterations=2000")
    rhs = O.box_rhs(N, 3, 3, 3, 7, el.get("ggeo"))
    x, info = el.solve(rhs)
    assert info["status"] == 0
    assert info["res"] <= 1e-8 * info["res0"]
    # true residual of the assembled system
    b = el.gs(el.mask(rhs))
    r = b - el.operator(x)
    w = el.get("invDegree")
    assert np.sqrt((w * r * r).sum() / el.volume) <= 2e-8 * info["res0"]


@pytest.mark.parametrize("form", ["projectionAconj", "projection"])
def test_oracle_solution_projection(oracle_mod, form):
    """Solution projection (ellipticSolutionProjection.cpp): right-hand sides drawn from a
    two-dimensional space are solved from the projected initial guess in a few iterations once
    the basis holds two solutions; every solve still meets the absolute tolerance."""
    VX, EToV, EToB = O.box_mesh(3, 3, 3, 0.3)
    N = 4
    base = "preconditioner=jacobi;solver=pcg;residualTol=1e-9;maxIterations=2000"
    plain = O.Elliptic(N, VX, EToV, EToB, base)
    proj = O.Elliptic(N, VX, EToV, EToB, base + f";initialGuess={form};residualProjectionVectors=4;"
                      "residualProjectionStart=2")
    b1 = O.box_rhs(N, 3, 3, 3, 7, plain.get("ggeo"))
    b2 = O.box_rhs(N, 3, 3, 3, 8, plain.get("ggeo"))
    w = plain.get("invDegree")
    its_plain, its_proj = [], []
    for k in range(6):
        rhs = np.cos(0.4 * k) * b1 + np.sin(0.4 * k) * b2
        x0, i0 = plain.solve(rhs)
        x1, i1 = proj.solve(rhs)
        assert i0["status"] == 0 and i1["status"] == 0
        its_plain.append(i0["iterations"])
        its_proj.append(i1["iterations"])
        b = plain.gs(plain.mask(rhs))
        r = b - plain.operator(x1)
        assert np.sqrt((w * r * r).sum() / plain.volume) <= 2e-9
        assert np.linalg.norm(x1 - x0) <= 1e-6 * np.linalg.norm(x0)
    assert its_proj[0] == its_plain[0]  # projection starts at the second solve
    assert max(its_proj[3:]) < min(its_plain) // 3, (its_plain, its_proj)


def test_oracle_block_helmholtz_sanity(oracle_mod):
    """Block / stress restatement: one field with scalar coefficients is the scalar Helmholtz operator
    (reference operation order) bit for bit; constant coefficient arrays equal the scalars; the stress operator annihilates a rigid
    rotation and is symmetric; its PCG converges."""
    N, n = 4, 3
    VX, EToV, EToB = O.box_mesh(n, n, n, 0.3)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    hel = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi;lambda0=1.3;lambda1=0.7;poisson=0")
    Nl = el.get("invDegree").size
    rng = np.random.default_rng(0)
    q = rng.standard_normal(Nl)
    b = el.block_ax(q, nf=1, l0=1.3, l1=0.7)
    assert np.array_equal(b, hel.ax_ref(q))
    assert np.array_equal(el.block_ax(q, nf=1, lam0=np.full(Nl, 1.3), lam1=np.full(Nl, 0.7)), b)
    # the scalar FP64 diagonal is formed in the device's fused order: equal to rounding
    assert np.allclose(el.block_inv_diag(nf=1, l0=1.3, l1=0.7), hel.get("invDiag"), rtol=1e-14, atol=0)
    x, y = el.get("x"), el.get("y")
    rot = np.concatenate([y, -x, np.zeros_like(x)])
    assert np.abs(el.block_ax(rot, nf=3, stress=True, l0=1.0, l1=0.0)).max() < 1e-12
    u, v = rng.standard_normal(3 * Nl), rng.standard_normal(3 * Nl)
    Au, Av = el.block_ax(u, nf=3, stress=True, l1=0.5), el.block_ax(v, nf=3, stress=True, l1=0.5)
    assert abs(v @ Au - u @ Av) < 1e-12 * abs(v @ Au)
    rhs = np.concatenate([O.box_rhs(N, n, n, n, s, el.get("ggeo")) for s in (1, 2, 3)])
    _, info = el.block_solve(rhs, nf=3, stress=True, l0=1.0, l1=10.0, tol=1e-8)
    assert info["status"] == 0 and info["res"] <= 1e-8 * info["res0"]


@pytest.mark.parametrize("precon", ["jacobi", "multigrid"])
def test_oracle_all_neumann_null_space(oracle_mod, precon):
    """All-Neumann Poisson (no Dirichlet face): the oracle detects the null space, removes the mean as
    ellipticZeroMean does, converges, and returns a zero-mean solution of the projected system."""
    N, n = 4, 3
    VX, EToV, EToB = O.box_mesh(n, n, n, 0.3, all_dirichlet=False)
    opts = (f"preconditioner={precon};solver=pfcg;residualTol=1e-10+relative;maxIterations=3000;"
            "pMGSchedule=p=4+degree=2,p=1,p=4+degree=2;smootherType=cheby+asm;mgPrecision=fp64")
    el = O.Elliptic(N, VX, EToV, EToB, opts)
    assert el.get("allNeumann")[0] == 1
    rhs = O.box_rhs(N, n, n, n, 5, el.get("ggeo")) + 1e-3
    x, info = el.solve(rhs)
    assert info["status"] == 0
    assert abs(x.sum()) <= 1e-12 * np.abs(x).sum()
    b = rhs - rhs.mean()
    r = el.gs(b) - el.operator(x)
    w = el.get("invDegree")
    assert np.sqrt((w * r * r).sum() / el.volume) <= 1e-9 * info["res0"] * 10
    dirichlet = O.Elliptic(N, VX, EToV, np.where(EToB > 0, 1, 0).astype(np.int32), opts)
    assert dirichlet.get("allNeumann")[0] == 0


def _ref_block(kind, lam, N, E, geo, D, q, l0, l1, loffset):
    import ctypes

    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    f = getattr(O.ref_lib(), f"ref_{kind}_N{N}" if lam is None else f"ref_{kind}_l{lam}_N{N}")
    Nq = N + 1
    DT = np.ascontiguousarray(D.reshape(Nq, Nq).T).ravel()
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = np.zeros_like(q)
    el = np.arange(E, dtype=np.int32)
    cE, off, lo = ctypes.c_int(E), ctypes.c_int(E * Nq ** 3), ctypes.c_int(loffset)
    f(ctypes.byref(cE), ctypes.byref(off), ctypes.byref(lo), P(el), P(np.ascontiguousarray(geo)),
      P(np.ascontiguousarray(D)), P(DT), P(np.ascontiguousarray(l0)), P(np.ascontiguousarray(l1)), P(q), P(out))
    return out


@pytest.mark.skipif(O.ref_lib() is None or not hasattr(O.ref_lib(), "ref_block_l1_N3"),
                    reason="reference kernels (oracle/_ref) not built on this host")
@pytest.mark.parametrize("N", [1, 3, 5, 7])
@pytest.mark.parametrize("kind", ["block", "stress"])
def test_oracle_block_operators_bitexact_vs_reference(oracle_mod, N, kind):
    """The oracle's block and stress axhelm against the reference's own serial kernels
    (ellipticBlockPartialAxCoeffHex3D.c, ellipticStressPartialAxCoeffHex3D.c), compiled from its sources:
    per-field coefficient fields (p_lambda 1, loffset = fieldOffset) and scalars (p_lambda 0)."""
    VX, EToV, EToB = O.box_mesh(2, 2, 1, 0.4)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=none")
    n = el.get("invDegree").size
    rng = np.random.default_rng(N)
    q = rng.uniform(-1, 1, 3 * n)
    lam0 = rng.uniform(0.5, 2.0, 3 * n)
    lam1 = rng.uniform(0.0, 3.0, 3 * n)
    geo = el.get("ggeo") if kind == "block" else el.block_vgeo()
    D = el.get("D")
    stress = kind == "stress"
    ref = _ref_block(kind, 1, N, VX.shape[0], geo, D, q, lam0, lam1, n)
    got = el.block_ax(q, nf=3, stress=stress, lam0=lam0, lam1=lam1, loffset=n)
    assert np.array_equal(got, ref)
    ref = _ref_block(kind, 0, N, VX.shape[0], geo, D, q, np.array([1.3]), np.array([0.7]), 0)
    got = el.block_ax(q, nf=3, stress=stress, l0=1.3, l1=0.7)
    assert np.array_equal(got, ref)


@pytest.mark.skipif(O.ref_lib() is None or not hasattr(O.ref_lib(), "ref_axcoef_N3"),
                    reason="reference kernels (oracle/_ref) not built on this host")
@pytest.mark.parametrize("N", [1, 3, 5, 7])
def test_oracle_coefficient_field_axhelm_bitexact_vs_reference(oracle_mod, N):
    """One field with per-node lambda0 / lambda1 (the p_lambda = 1 build of ellipticPartialAxCoeffHex3D.c,
    a scalar Helmholtz solve with coefficient fields) against the oracle's block operator with nf = 1."""
    VX, EToV, EToB = O.box_mesh(2, 1, 2, 0.4)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=none")
    n = el.get("invDegree").size
    rng = np.random.default_rng(10 + N)
    q, lam0, lam1 = rng.uniform(-1, 1, n), rng.uniform(0.5, 2.0, n), rng.uniform(0.0, 3.0, n)
    ref = _ref_block("axcoef", None, N, VX.shape[0], el.get("ggeo"), el.get("D"), q, lam0, lam1, 0)
    got = el.block_ax(q, nf=1, lam0=lam0, lam1=lam1)
    assert np.array_equal(got, ref)


def test_oracle_trilinear_lambda0_on_t_flux_only(oracle_mod):
    """The reference's trilinear kernel scales the t-flux alone by lambda0 (ellipticPartialAxTrilinearHex3D.okl:
    154-157); option trilinearLambda0=all scales all three.  On an undeformed box a field that does not vary in
    z has no t-flux, so the default operator ignores lambda0 there, while the all-flux form scales by it."""
    N, n = 4, 2
    VX, EToV, EToB = O.box_mesh(n, n, n, 1.0)  # Kershaw eps = 1: the undeformed box
    base = "preconditioner=jacobi;elementMap=trilinear"
    a1 = O.Elliptic(N, VX, EToV, EToB, base)
    a2 = O.Elliptic(N, VX, EToV, EToB, base + ";lambda0=2.5")
    a3 = O.Elliptic(N, VX, EToV, EToB, base + ";lambda0=2.5;trilinearLambda0=all")
    x, y = a1.get("x"), a1.get("y")
    q = np.sin(2.0 * x) * np.cos(3.0 * y)
    r1, r2, r3 = a1.ax(q), a2.ax(q), a3.ax(q)
    scale = np.max(np.abs(r1))
    assert np.max(np.abs(r2 - r1)) <= 1e-13 * scale
    assert np.max(np.abs(r3 - 2.5 * r1)) <= 1e-13 * scale
    # a field varying in z only: the t-flux is all there is, both forms scale it
    zc = a1.get("z")
    qz = np.cos(2.0 * zc)
    assert np.max(np.abs(a2.ax(qz) - 2.5 * a1.ax(qz))) <= 1e-13 * np.max(np.abs(a1.ax(qz)))


def test_oracle_config0_matches_fixture(oracle_mod):
    """The oracle's E=8^3 Jacobi-PCG solve reproduces the committed fixture (iterations, history, solution)."""
    import hashlib
    import json

    from nekrs_gb300 import workloads as W

    with open(os.path.join(os.path.dirname(__file__), "golden", "config_parity.json")) as f:
        cfg = json.load(f)["c0"]
    VX, EToV, EToB = W.kershaw_box(cfg["nel"], eps=cfg["eps"])
    orc = O.Elliptic(cfg["N"], VX, EToV, EToB, cfg["options"])
    x, io = orc.solve(W.box_rhs(cfg["N"], cfg["nel"], cfg["nel"], cfg["nel"], cfg["seed"], orc.get("ggeo")))
    assert io["iterations"] == cfg["iterations"]
    assert np.allclose(io["history"], cfg["history"], rtol=1e-10, atol=0)
    assert abs(np.linalg.norm(x) - cfg["x_norm"]) <= 1e-12 * cfg["x_norm"]
    assert hashlib.sha256(x.tobytes()).hexdigest() == cfg["x_sha256"]
