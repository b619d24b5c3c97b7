"""The FDM (Schwarz local solve) in TF32 on the tensor cores
(fdmPrecision = tf32): mma.sync m16n8k8 transforms with TF32 inputs and FP32
accumulation, no scaling.  Checked against the FP32 kernels on the same level
data for orders 7, 5 and 3, RAS and ASM (TF32 has an 11-bit significand: the
bar is 1e-2 of max |Su|; measured values are printed), and end to end: the
mixed-precision solve with the TF32 smoother meets its tolerance, takes about
as many iterations as the FP32 smoother and stays within 1e-8 of the
FP64-throughout oracle."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SCHED = {7: "p=7+degree=5,p=3+degree=5,p=1,p=3+degree=5,p=7+degree=5",
         5: "p=5+degree=5,p=3+degree=5,p=1,p=3+degree=5,p=5+degree=5"}


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("schwarz", ["ras", "asm"])
@pytest.mark.parametrize("N,level", [(7, 0), (7, 1), (5, 0)])
@pytest.mark.parametrize("eps", [0.3, 1.0])
def test_fdm_tf32_matches_fp32(product_lib, torch_cuda, N, level, schwarz, eps):
    torch = torch_cuda
    n = 4
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    base = (f"solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+{schwarz};maxIterations=200;"
            f"pMGSchedule={SCHED[N]};coarseSolver=jpcg;coarseTol=1e-4;mgPrecision=mixed")
    e32 = G.Elliptic(N, VX, EToV, EToB, base + ";fdmPrecision=fp32")
    etf = G.Elliptic(N, VX, EToV, EToB, base + ";fdmPrecision=tf32")
    m = e32.mg_level_size(level)
    u = torch.from_numpy(np.random.default_rng(5).uniform(-1, 1, m).astype(np.float32)).cuda()
    s32, stf = torch.zeros_like(u), torch.zeros_like(u)
    e32.mg_fdm(level, u, s32)
    etf.mg_fdm(level, u, stf)
    torch.cuda.synchronize()
    a, b = s32.cpu().numpy().astype(np.float64), stf.cpu().numpy().astype(np.float64)
    err = np.max(np.abs(a - b)) / np.max(np.abs(a))
    print(f"TF32 FDM vs FP32 FDM (N={N} level {level} {schwarz} eps={eps}): max error {err:.2e} of max |Su|, "
          f"rel 2-norm {rel(b, a):.2e}")
    assert np.isfinite(b).all()
    assert err < 1e-2


@pytest.mark.parametrize("eps", [0.3, 1.0])
def test_fdm_tcgen05_matches_mma_sync(product_lib, torch_cuda, eps):
    """The order-7 RAS FDM on tcgen05.mma (the default for fdmPrecision = tf32) against the mma.sync form of the
    same TF32 transforms and against the FP32 kernel; E = 2^3 and 5^3 (every persistent CTA takes at most one
    element and prefetches no next one: the grid, SMs x resident CTAs, is larger than E) and E = 12^3 (several
    elements per CTA)."""
    torch = torch_cuda
    N = 7
    for n in (2, 5, 12):
        VX, EToV, EToB = W.kershaw_box(n, eps=eps)
        base = (f"solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+ras;maxIterations=200;"
                f"pMGSchedule={SCHED[N]};coarseSolver=jpcg;coarseTol=1e-4;mgPrecision=mixed")
        out = {}
        for name, o in (("fp32", ";fdmPrecision=fp32"), ("sync", ";fdmPrecision=tf32;fdmMma=sync"),
                        ("tcgen05", ";fdmPrecision=tf32;fdmMma=tcgen05")):
            el = G.Elliptic(N, VX, EToV, EToB, base + o)
            m = el.mg_level_size(0)
            u = torch.from_numpy(np.random.default_rng(9).uniform(-1, 1, m).astype(np.float32)).cuda()
            su = torch.full_like(u, float("nan"))
            el.mg_fdm(0, u, su)
            torch.cuda.synchronize()
            out[name] = su.cpu().numpy().astype(np.float64)
            del el
        a = out["fp32"]
        for name in ("sync", "tcgen05"):
            err = np.max(np.abs(out[name] - a)) / np.max(np.abs(a))
            print(f"E={n}^3 eps={eps}: {name} TF32 FDM vs FP32: max error {err:.2e} of max |Su|")
            assert np.isfinite(out[name]).all()
            assert err < 1e-2
        d = np.max(np.abs(out["tcgen05"] - out["sync"])) / np.max(np.abs(a))
        print(f"E={n}^3 eps={eps}: tcgen05 vs mma.sync: {d:.2e}")
        assert d < 2e-3


@pytest.mark.parametrize("schwarz", ["ras", "asm"])
def test_mixed_tf32_smoother_solve(product_lib, oracle_mod, torch_cuda, schwarz):
    torch = torch_cuda
    n, N = 4, 7
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = (f"solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+{schwarz};maxIterations=200;"
            f"pMGSchedule={SCHED[N]};coarseSolver=jpcg;coarseTol=1e-4;residualTol=1e-8+relative")
    orc = O.Elliptic(N, VX, EToV, EToB, opts + ";mgPrecision=fp64")
    rhs = W.box_rhs(N, n, n, n, 7, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    its, xs = {}, {}
    for prec in ("fp32", "tf32"):
        el = G.Elliptic(N, VX, EToV, EToB, opts + f";mgPrecision=mixed;fdmPrecision={prec}")
        r = torch.from_numpy(rhs.copy()).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        assert info["status"] == 0 and info["res"] <= 1e-8 * info["res0"]
        its[prec], xs[prec] = info["iterations"], x.cpu().numpy()
    print(f"iterations ({schwarz}): oracle FP64 {io['iterations']}, mixed FP32 FDM {its['fp32']}, "
          f"mixed TF32 FDM {its['tf32']}; error vs FP64 oracle {rel(xs['tf32'], xo):.2e}")
    assert its["tf32"] <= its["fp32"] + 2
    assert rel(xs["tf32"], xo) < 1e-8
