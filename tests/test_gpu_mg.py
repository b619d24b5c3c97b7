"""p-multigrid parity on the GPU against the CPU oracle.

FP64 multigrid (mgPrecision=fp64, the plain form): same lambda_max estimates
(1e-9 relative), same iteration counts, solutions within 1e-10 relative.
FP32 multigrid (the reference's pfloat default): iteration counts within one,
converged to the tolerance, solution within 1e-7 of the FP64 oracle solve."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SCHED = {7: "p=7+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=7+degree=2",
         5: "p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=5+degree=2",
         3: "p=3+degree=2,p=1,p=3+degree=2"}


def solve_both(torch, N, n, opts, eps=0.3, seed=3):
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    rhs = W.box_rhs(N, n, n, n, seed, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    torch.cuda.synchronize()
    return orc, el, xo, io, x.cpu().numpy(), ig, rhs


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("smoother,solver", [("cheby+jac", "pcg"), ("cheby+asm", "pcg"), ("fourthcheby+asm", "pcg"),
                                             ("fourthoptcheby+asm", "pcg"), ("cheby+ras", "pfcg"),
                                             ("fourthoptcheby+ras", "pfgmres")])
@pytest.mark.parametrize("N", [3, 7])
def test_mg_fp64_parity(product_lib, oracle_mod, torch_cuda, smoother, solver, N):
    opts = (f"solver={solver};preconditioner=multigrid;smootherType={smoother};mgPrecision=fp64;"
            f"residualTol=1e-8+relative;maxIterations=200;pMGSchedule={SCHED[N]}")
    orc, el, xo, io, xg, ig, _ = solve_both(torch_cuda, N, 3, opts)
    assert np.allclose(el.get("mg.rho"), orc.mg_info("rho"), rtol=1e-9, atol=0)
    assert list(el.get("mg.levels")) == list(orc.mg_info("levels"))
    assert ig["status"] == 0 and io["status"] == 0
    assert ig["iterations"] == io["iterations"]
    assert rel(xg, xo) < 1e-10


@pytest.mark.parametrize("smoother,solver", [("cheby+asm", "pcg"), ("fourthoptcheby+ras", "pfcg")])
def test_mg_fp32_matches_fp64_oracle(product_lib, oracle_mod, torch_cuda, smoother, solver):
    N, n = 7, 3
    base = (f"solver={solver};preconditioner=multigrid;smootherType={smoother};residualTol=1e-8+relative;"
            f"maxIterations=200;pMGSchedule={SCHED[N]}")
    orc32, el, xo32, io32, xg, ig, rhs = solve_both(torch_cuda, N, n, base + ";mgPrecision=fp32")
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    orc64 = O.Elliptic(N, VX, EToV, EToB, base + ";mgPrecision=fp64")
    xo64, io64 = orc64.solve(rhs)
    assert np.allclose(el.get("mg.rho"), orc32.mg_info("rho"), rtol=1e-4)
    assert abs(ig["iterations"] - io32["iterations"]) <= 1
    assert ig["res"] <= 1e-8 * ig["res0"]
    assert rel(xg, xo64) < 1e-7


def test_default_levels_and_smoothed_coarse(product_lib, oracle_mod, torch_cuda):
    # Chebyshev+Jacobi default levels for N=7 are 7,5,3,1 (determineMGLevels.cpp:81-96)
    opts = ("solver=pcg;preconditioner=multigrid;smootherType=cheby+jac;mgPrecision=fp64;coarseSolver=smooth;"
            "residualTol=1e-8+relative;maxIterations=300")
    orc, el, xo, io, xg, ig, _ = solve_both(torch_cuda, 7, 2, opts)
    assert list(el.get("mg.levels")) == [7, 5, 3, 1]
    assert ig["iterations"] == io["iterations"]
    assert rel(xg, xo) < 1e-10


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
@pytest.mark.parametrize("smoother", ["cheby+asm", "cheby+ras"])
@pytest.mark.parametrize("N", [2, 5, 7])
def test_schwarz_smoother_parity(product_lib, oracle_mod, torch_cuda, smoother, N, prec, tol):
    """One application of the level-0 Schwarz smoother against the FP64 oracle (FP32 multigrid: within FP32
    rounding of the six 1-D transforms; order 7 in FP32 runs the warp-per-element kernel)."""
    torch = torch_cuda
    n = 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.5)
    sched = f"p={N}+degree=2,p=1,p={N}+degree=2"
    opts = (f"solver=pfcg;preconditioner=multigrid;smootherType={smoother};mgPrecision=fp64;pMGSchedule={sched}")
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    opts = opts.replace("mgPrecision=fp64", f"mgPrecision={prec}")
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    u = np.random.default_rng(N).uniform(-1, 1, orc.Nlocal)
    u = orc.mask(orc.gs(u) * orc.get("invDegree"))  # a continuous, masked field
    ref = orc.mg_schwarz(0, u)
    ud = torch.from_numpy(u).cuda()
    out = torch.zeros_like(ud)
    el.mg_smoother(0, ud, out)
    assert np.max(np.abs(out.cpu().numpy() - ref)) < tol * np.max(np.abs(ref))


def test_persistent_coarse_matches_host_driven(product_lib, torch_cuda):
    """The cooperative coarse Jacobi-PCG gives the same preconditioner as the host-driven loop."""
    torch = torch_cuda
    N, n = 5, 4
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    base = (f"solver=pfcg;preconditioner=multigrid;smootherType=cheby+asm;mgPrecision=fp64;"
            f"residualTol=1e-9+relative;maxIterations=200;pMGSchedule={SCHED[5]}")
    sols, its = [], []
    for pers in (1, 0):
        el = G.Elliptic(N, VX, EToV, EToB, base + f";coarsePersistent={pers}")
        rhs = W.box_rhs(N, n, n, n, 8, el.get("ggeo"))
        r = torch.from_numpy(rhs).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        assert info["status"] == 0
        its.append(info["iterations"])
        sols.append(x.cpu().numpy())
        assert el.get("mg.coarseError")[0] == 0
        if pers:
            # the persistent solve runs on the assembled order-1 operator: one row per unmasked unique node
            rows, width, nnz, grid, chunk, in_smem, cluster = el.get("mg.coarseMatrix")
            assert rows == (n - 1) ** 3 and 7 <= width <= 27 and rows <= nnz <= rows * width
            assert grid * chunk >= rows and in_smem == 1
        else:
            assert len(el.get("mg.coarseMatrix")) == 0
    assert its[0] == its[1]
    assert rel(sols[0], sols[1]) < 1e-10


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("n", [20, 36])
def test_persistent_coarse_many_row_blocks(product_lib, torch_cuda, prec, n):
    """A coarse level spread over several CTAs (row blocks with halos, grid barriers between them) gives the
    same preconditioner as the host-driven coarse loop on the E-vector level operator: 19^3 = 6859 rows as
    one thread-block cluster of 2 CTAs (hardware cluster barrier), 35^3 = 42875 rows over many CTAs of a
    cooperative launch (counting grid barrier)."""
    torch = torch_cuda
    N = 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    base = (f"solver=pfcg;preconditioner=multigrid;smootherType=cheby+asm;mgPrecision={prec};"
            f"residualTol=1e-9+relative;maxIterations=200;pMGSchedule={SCHED[3]}")
    sols, its, cits = [], [], []
    for pers in (1, 0):
        el = G.Elliptic(N, VX, EToV, EToB, base + f";coarsePersistent={pers}")
        if pers:
            rows, width, nnz, grid, chunk, in_smem, cluster = el.get("mg.coarseMatrix")
            assert rows == (n - 1) ** 3
            if n == 20:
                assert grid == 2 and cluster == 2
            else:
                assert grid >= 8 and cluster == 0
        rhs = W.box_rhs(N, n, n, n, 11, el.get("ggeo"))
        r = torch.from_numpy(rhs).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        assert info["status"] == 0
        its.append(info["iterations"])
        cits.append(el.get("mg.coarseIters")[-1])
        sols.append(x.cpu().numpy())
        assert el.get("mg.coarseError")[0] == 0
    if prec == "fp64":
        assert its[0] == its[1] and abs(cits[0] - cits[1]) <= 1
        assert rel(sols[0], sols[1]) < 1e-10
    else:
        assert abs(its[0] - its[1]) <= 1 and abs(cits[0] - cits[1]) <= 3
        assert rel(sols[0], sols[1]) < 1e-7


def test_mixed_precision_error_vs_fp64_oracle(product_lib, oracle_mod, torch_cuda):
    """mgPrecision=mixed: FP32 multigrid under the FP64-accurate FP32-pair fine operator; the error
    against the FP64-throughout oracle solve is at the level the tolerance allows (1e-8 here)."""
    N, n = 7, 3
    base = (f"solver=pfcg;preconditioner=multigrid;smootherType=cheby+asm;residualTol=1e-10+relative;"
            f"maxIterations=200;pMGSchedule={SCHED[7]}")
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    orc = O.Elliptic(N, VX, EToV, EToB, base + ";mgPrecision=fp64")
    rhs = W.box_rhs(N, n, n, n, 5, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    el = G.Elliptic(N, VX, EToV, EToB, base + ";mgPrecision=mixed")
    torch = torch_cuda
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    assert ig["status"] == 0
    assert ig["res"] <= 1e-10 * ig["res0"]
    assert abs(ig["iterations"] - io["iterations"]) <= 2
    assert rel(x.cpu().numpy(), xo) < 1e-8


@pytest.mark.parametrize("N", [3, 7])
def test_fdm_entry_point_matches_smoother(product_lib, torch_cuda, N):
    """RAS: one launch of the fused FDM entry point followed by gather-scatter and mask (done here on the
    host in FP32, member order) equals the level-0 Schwarz smoother, bit for bit."""
    torch = torch_cuda
    n = 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.5)
    opts = (f"solver=pfcg;preconditioner=multigrid;smootherType=cheby+ras;mgPrecision=fp32;"
            f"pMGSchedule=p={N}+degree=2,p=1,p={N}+degree=2")
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    assert el.get("mg.bytes")[0] == 4
    m = el.mg_level_size(0)
    u = np.random.default_rng(N).uniform(-1, 1, m).astype(np.float32)
    ud = torch.from_numpy(u).cuda()
    su = torch.zeros_like(ud)
    el.mg_fdm(0, ud, su)
    torch.cuda.synchronize()
    s = su.cpu().numpy()
    off, ids = el.get("gsOff"), el.get("gsIds")
    out = s.copy()
    for g in range(len(off) - 1):
        mem = ids[off[g]:off[g + 1]]
        if len(mem) > 1:
            v = np.float32(0)
            for k in mem:
                v = np.float32(v + s[k])
            out[mem] = v
    out[el.get("maskIds")] = 0
    ref = torch.zeros(m, dtype=torch.float64, device="cuda")
    el.mg_smoother(0, torch.from_numpy(u.astype(np.float64)).cuda(), ref)
    assert np.array_equal(out.astype(np.float64), ref.cpu().numpy())


@pytest.mark.parametrize("disc", ["fem+galerkin", "semfem"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_mg_galerkin_coarse_operator_parity(product_lib, oracle_mod, torch_cuda, prec, disc):
    """coarseGridDiscretization = FEM+Galerkin (B^T A_fine B) or SEMFEM (linear tetrahedra on the order-1
    grid): the persistent coarse Jacobi-PCG runs on the operator built on the host (equal to the oracle's);
    the V-cycle solve matches the oracle's."""
    opts = (f"solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+asm;mgPrecision={prec};"
            f"residualTol=1e-8+relative;maxIterations=200;pMGSchedule={SCHED[5]};coarseGridDiscretization={disc}")
    orc, el, xo, io, xg, ig, _ = solve_both(torch_cuda, 5, 4, opts)
    assert ig["status"] == 0 and io["status"] == 0
    assert abs(ig["iterations"] - io["iterations"]) <= 1
    assert ig["res"] <= 1e-8 * ig["res0"]
    assert rel(xg, xo) < (1e-8 if prec == "fp64" else 1e-6)


@pytest.mark.parametrize("N", [5, 7])
def test_axhelm_autotuner(product_lib, torch_cuda, N):
    """The setup-time autotuner times the interchangeable FP32 axhelm variants of every smoothed level on the
    level's own data, keeps only those bit-identical to the default kernel, and picks the fastest; the solve
    with the tuned choice is bit-identical to the solve with the default kernel forced."""
    torch = torch_cuda
    n = 5
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    sched = f"p={N}+degree=3,p=3+degree=3,p=1,p=3+degree=3,p={N}+degree=3"
    base = ("solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+ras;mgPrecision=mixed;"
            f"residualTol=1e-9+relative;maxIterations=100;pMGSchedule={sched}")
    sols = []
    for kern in ("auto", "vec"):
        el = G.Elliptic(N, VX, EToV, EToB, base + f";axKernel={kern}")
        chosen = el.get("mg.axKernel")
        times = el.get("mg.axTimes").reshape(len(chosen), 6)
        if kern == "auto":
            assert (times[:, 0] > 0).all() and (times[:, 1] > 0).all()  # default and plain always apply
            if N == 7:
                assert (times[0] > 0).sum() >= 5                          # vec, plain, epb2, const, constpf
            for lvl, c in enumerate(chosen.astype(int)):
                ok = times[lvl] > 0
                assert ok[c] and times[lvl, c] == times[lvl][ok].min()
        else:
            assert (chosen == 0).all()
        rhs = W.box_rhs(N, n, n, n, 9, el.get("ggeo"))
        r = torch.from_numpy(rhs).cuda()
        x = torch.zeros_like(r)
        assert el.solve(r, x)["status"] == 0
        sols.append(x.cpu().numpy())
    assert np.array_equal(sols[0], sols[1])
