"""End-to-end solve parity: the GPU ellipticSolve against the CPU oracle on the
same Kershaw boxes and seeded right-hand sides.  Bar for the plain FP64 form
(stored geometry, Jacobi or no preconditioner, every Krylov variant):
bit-identical -- the same iteration count, the same residual history and the
same solution, bit for bit.  Finite-precision CG amplifies any rounding
difference (a 1e-16 change of the right-hand side moves Jacobi-PCG's count by
one and its solution by ~1e-9 at a 1e-8 tolerance), so only identical
arithmetic gives the north star's "identical iteration counts, 1e-10"
reliably; the device and the oracle share the reduction order and the fused
multiply-add placement for that reason."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run_pair(torch, N, n, opts, eps=0.3, seed=11, x0=None):
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    rhs = W.box_rhs(N, n, n, n, seed, orc.get("ggeo"))
    xo, io = orc.solve(rhs, x0)
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r) if x0 is None else torch.from_numpy(x0.copy()).cuda()
    ig = el.solve(r, x)
    torch.cuda.synchronize()
    return xo, io, x.cpu().numpy(), ig, el, orc


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def assert_bit_identical(xo, io, xg, ig, el):
    assert ig["status"] == io["status"]
    assert ig["iterations"] == io["iterations"]
    assert ig["res0"] == io["res0"] and ig["res"] == io["res"]
    assert np.array_equal(el.get("history"), np.asarray(io["history"]))
    assert np.array_equal(xg, xo)


@pytest.mark.parametrize("N,n", [(1, 4), (3, 3), (5, 3), (7, 3), (9, 2)])
def test_jacobi_pcg_parity(product_lib, oracle_mod, torch_cuda, N, n):
    """Jacobi-PCG (70-150 iterations here): bit-identical to the oracle."""
    opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=3000"
    xo, io, xg, ig, el, orc = run_pair(torch_cuda, N, n, opts)
    assert ig["status"] == 0
    assert_bit_identical(xo, io, xg, ig, el)


@pytest.mark.parametrize("solver", ["pfcg", "pgmres+nVector=10", "pfgmres", "pcg;preconditioner=none"])
def test_krylov_variants_parity(product_lib, oracle_mod, torch_cuda, solver):
    opts = f"preconditioner=jacobi;solver={solver};residualTol=1e-8+relative;maxIterations=3000"
    xo, io, xg, ig, el, orc = run_pair(torch_cuda, 4, 3, opts)
    assert ig["status"] == 0
    assert_bit_identical(xo, io, xg, ig, el)


def test_nonzero_initial_guess_and_helmholtz(product_lib, oracle_mod, torch_cuda):
    N, n = 4, 3
    opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-9+relative;poisson=0;lambda0=1.0;lambda1=2.5"
    rng = np.random.default_rng(5)
    x0 = rng.uniform(-1, 1, n ** 3 * (N + 1) ** 3)
    xo, io, xg, ig, el, orc = run_pair(torch_cuda, N, n, opts, x0=x0)
    assert_bit_identical(xo, io, xg, ig, el)


@pytest.mark.parametrize("lam", ["", ";trilinearLambda0=all"])
def test_trilinear_operator_solve(product_lib, oracle_mod, torch_cuda, lam):
    """Recomputed (trilinear) geometry, Helmholtz with lambda0 != 1 on the reference's t-flux-only scaling and
    on the all-flux option: bit-identical to the oracle."""
    opts = ("preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;elementMap=trilinear;poisson=0;"
            "lambda0=1.4;lambda1=0.3" + lam)
    xo, io, xg, ig, el, orc = run_pair(torch_cuda, 5, 3, opts, eps=1.0)
    assert ig["status"] == 0
    assert_bit_identical(xo, io, xg, ig, el)


def test_operator_gs_mask_entry_points(product_lib, oracle_mod, torch_cuda):
    torch = torch_cuda
    N, n = 6, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = "preconditioner=jacobi"
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    q = np.random.default_rng(2).uniform(-1, 1, orc.Nlocal)
    qd = torch.from_numpy(q).cuda()
    out = torch.zeros_like(qd)
    el.operator(qd, out)
    ref = orc.operator(q)
    assert np.array_equal(out.cpu().numpy(), ref)
    for k in ("ids", "gsOff", "gsIds", "maskIds", "invDegree", "ggeo", "invDiag", "D"):
        assert np.array_equal(el.get(k), orc.get(k)), k


def test_host_buffer_solve_matches_device_solve(product_lib, torch_cuda):
    torch = torch_cuda
    N, n = 5, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = "preconditioner=jacobi;residualTol=1e-8+relative"
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    g = el.get("ggeo")
    rhs = W.box_rhs(N, n, n, n, 3, g)
    r1, x1 = rhs.copy(), np.zeros_like(rhs)
    i1 = el.solve_host(r1, x1)
    r2 = torch.from_numpy(rhs.copy()).cuda()
    x2 = torch.zeros_like(r2)
    i2 = el.solve(r2, x2)
    assert i1["iterations"] == i2["iterations"]
    assert np.array_equal(x1, x2.cpu().numpy())  # deterministic reductions


def test_status_codes(product_lib, torch_cuda):
    torch = torch_cuda
    N, n = 3, 2
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    el = G.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi;maxIterations=3;residualTol=1e-12+relative")
    rhs = W.box_rhs(N, n, n, n, 1, el.get("ggeo"))
    r = torch.from_numpy(rhs).cuda()
    x = torch.zeros_like(r)
    info = el.solve(r, x)
    assert info["status"] == 1 and info["iterations"] == 3  # MAXIT, not an abort
    bad = rhs.copy()
    bad[1 + 4 + 16] = np.nan  # node (1,1,1) of element 0: interior, not masked
    r = torch.from_numpy(bad).cuda()
    with pytest.raises(G.NrsgError) as e:
        el.solve(r, torch.zeros_like(r))
    assert e.value.code == 3
    # zero right-hand side: nothing to do
    r = torch.zeros(el.Nlocal, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(r)
    info = el.solve(r, x)
    assert info["iterations"] == 0 and float(x.abs().max()) == 0.0
    with pytest.raises(G.NrsgError) as e:
        G.Elliptic(N, VX, EToV, EToB, "preconditioner=bogus")
    assert e.value.code == 5


@pytest.mark.parametrize("precon", ["jacobi", "multigrid"])
def test_fp32x2_operator_solve_parity(product_lib, oracle_mod, torch_cuda, precon):
    """Solve with the FP32-pair fine operator against the FP64 oracle: same iterations, 1e-10."""
    extra = ";smootherType=cheby+asm;mgPrecision=fp64;pMGSchedule=p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=5+degree=2" \
        if precon == "multigrid" else ""
    base = f"preconditioner={precon};solver=pcg;residualTol=1e-8+relative;maxIterations=3000" + extra
    N, n = 5, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    orc = O.Elliptic(N, VX, EToV, EToB, base)
    rhs = W.box_rhs(N, n, n, n, 21, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    el = G.Elliptic(N, VX, EToV, EToB, base + ";axPrecision=fp32x2")
    torch = torch_cuda
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    assert ig["status"] == 0
    assert abs(ig["iterations"] - io["iterations"]) <= 1
    assert rel(x.cpu().numpy(), xo) < (1e-10 if precon == "multigrid" else 1e-8)


@pytest.mark.parametrize("z_bc", [1, 4])
def test_jacobi_pcg_parity_axis_fan(product_lib, oracle_mod, torch_cuda, z_bc):
    """A mesh that is not a box: twelve sectors around an axis in two layers (axis edges in 12 elements,
    the interior axis vertex in 24), Dirichlet outside, Dirichlet or Neumann ends.  The right-hand side is
    a smooth function of the node coordinates (continuous across elements) times JW; the GPU's Jacobi-PCG
    is bit-identical to the oracle's."""
    torch = torch_cuda
    N = 5
    VX, EToV, EToB = W.axis_fan(12, 2, z_bc=z_bc)
    opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-10+relative;maxIterations=3000"
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    x, y, z = orc.get("x"), orc.get("y"), orc.get("z")
    JW = orc.get("ggeo").reshape(len(EToV), 7, (N + 1) ** 3)[:, 6, :].ravel()
    rhs = (np.sin(3.0 * x + 0.5) * np.cos(2.0 * y) + z * z) * JW
    xo, io = orc.solve(rhs)
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    r = torch.from_numpy(rhs.copy()).cuda()
    xg = torch.zeros_like(r)
    ig = el.solve(r, xg)
    torch.cuda.synchronize()
    assert ig["status"] == 0
    assert_bit_identical(xo, io, xg.cpu().numpy(), ig, el)


def test_jacobi_pcg_parity_tight_tolerance(product_lib, oracle_mod, torch_cuda):
    """At a 1e-12 tolerance: still bit-identical."""
    opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-12+relative;maxIterations=3000"
    xo, io, xg, ig, el, orc = run_pair(torch_cuda, 5, 3, opts)
    assert_bit_identical(xo, io, xg, ig, el)


def test_solve_ordered_with_callers_torch_stream(product_lib, torch_cuda):
    """Buffers written on the caller's torch stream are read only after those writes: the right-hand side
    is copied in behind a GPU sleep on a side stream, right before the solve is called."""
    torch = torch_cuda
    N, n = 5, 4
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-10+relative;maxIterations=2000"
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    rhs = W.box_rhs(N, n, n, n, 21, el.get("ggeo"))
    rhs_d = torch.from_numpy(rhs).cuda()
    r = rhs_d.clone()
    x = torch.zeros_like(r)
    ref = el.solve(r, x)
    x_ref = x.cpu().numpy()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        r2 = torch.full_like(rhs_d, 1.0e3)
        x2 = torch.full_like(rhs_d, -7.0)
        torch.cuda._sleep(100_000_000)  # about 50 ms of GPU time before the writes below
        r2.copy_(rhs_d)
        x2.zero_()
        info = el.solve(r2, x2)
    side.synchronize()
    assert info["iterations"] == ref["iterations"]
    assert np.array_equal(x2.cpu().numpy(), x_ref)


@pytest.mark.parametrize("precon", ["jacobi", "multigrid"])
def test_all_neumann_poisson_parity(product_lib, oracle_mod, torch_cuda, precon):
    """Poisson with Neumann faces only (ellipticSetup.cpp:187-205): the constant null space is handled as the
    reference does (ellipticZeroMean on r, on every preconditioned z and on x); parity with the oracle."""
    torch = torch_cuda
    N, n = 5, 4
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3, all_dirichlet=False)
    if precon == "jacobi":
        opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=3000"
    else:
        opts = ("solver=pfcg;residualTol=1e-8+relative;maxIterations=200;preconditioner=multigrid;"
                "smootherType=fourthoptcheby+asm;pMGSchedule=p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,"
                "p=5+degree=2;mgPrecision=fp64")
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    rhs = W.box_rhs(N, n, n, n, 3, orc.get("ggeo")) + 1e-3  # a right-hand side with a nonzero mean
    xo, io = orc.solve(rhs)
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    assert el.get("allNeumann")[0] == 1 and orc.get("allNeumann")[0] == 1
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    torch.cuda.synchronize()
    xg = x.cpu().numpy()
    assert ig["status"] == 0 and io["status"] == 0
    assert abs(xg.sum()) <= 1e-12 * np.abs(xg).sum()
    if precon == "jacobi":
        assert_bit_identical(xo, io, xg, ig, el)
    else:  # FP64 multigrid: same iteration count, 1e-10
        assert ig["iterations"] == io["iterations"]
        assert abs(ig["res0"] - io["res0"]) <= 1e-12 * io["res0"]
        assert rel(xg, xo) < 1e-10
