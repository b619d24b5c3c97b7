"""The order-7 RAS FDM (Schwarz local solve) in FP16 on the tensor cores
(fdmPrecision = fp16): mma.sync m16n8k16 transforms, FP32 accumulation,
per-element max-abs scaling of the input, of each direction's eigenvector
matrix and of 1/(lx + ly + lz).  Checked against the FP32 kernel on the same
level data (FP16 has an 11-bit significand: the bar is 1e-2 of max |Su|,
measured values are printed), and end to end: the mixed-precision solve with
the FP16 smoother still meets its tolerance, takes about as many iterations
as the FP32 smoother and stays within 1e-8 of the FP64-throughout oracle."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SCHED7 = "p=7+degree=5,p=3+degree=5,p=1,p=3+degree=5,p=7+degree=5"
BASE = ("solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+ras;maxIterations=200;"
        f"pMGSchedule={SCHED7};coarseSolver=jpcg;coarseTol=1e-4")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("eps", [0.3, 1.0])
def test_fdm_fp16_matches_fp32(product_lib, torch_cuda, eps):
    torch = torch_cuda
    n, N = 4, 7
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    e32 = G.Elliptic(N, VX, EToV, EToB, BASE + ";mgPrecision=mixed;fdmPrecision=fp32")
    e16 = G.Elliptic(N, VX, EToV, EToB, BASE + ";mgPrecision=mixed;fdmPrecision=fp16")
    m = e32.mg_level_size(0)
    u = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, m).astype(np.float32)).cuda()
    s32, s16 = torch.zeros_like(u), torch.zeros_like(u)
    e32.mg_fdm(0, u, s32)
    e16.mg_fdm(0, u, s16)
    torch.cuda.synchronize()
    a, b = s32.cpu().numpy().astype(np.float64), s16.cpu().numpy().astype(np.float64)
    err = np.max(np.abs(a - b)) / np.max(np.abs(a))
    print(f"FP16 FDM vs FP32 FDM (eps={eps}): max error {err:.2e} of max |Su|, rel 2-norm {rel(b, a):.2e}")
    assert np.isfinite(b).all()
    assert err < 1e-2


def test_mixed_fp16_smoother_solve(product_lib, oracle_mod, torch_cuda):
    torch = torch_cuda
    n, N = 4, 7
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = BASE + ";residualTol=1e-8+relative"
    orc = O.Elliptic(N, VX, EToV, EToB, opts + ";mgPrecision=fp64")
    rhs = W.box_rhs(N, n, n, n, 7, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    its, xs = {}, {}
    for prec in ("fp32", "fp16"):
        el = G.Elliptic(N, VX, EToV, EToB, opts + f";mgPrecision=mixed;fdmPrecision={prec}")
        r = torch.from_numpy(rhs.copy()).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        assert info["status"] == 0 and info["res"] <= 1e-8 * info["res0"]
        its[prec], xs[prec] = info["iterations"], x.cpu().numpy()
    print(f"iterations: oracle FP64 {io['iterations']}, mixed FP32 FDM {its['fp32']}, mixed FP16 FDM {its['fp16']}; "
          f"error vs FP64 oracle {rel(xs['fp16'], xo):.2e}")
    assert its["fp16"] <= its["fp32"] + 2
    assert rel(xs["fp16"], xo) < 1e-8
