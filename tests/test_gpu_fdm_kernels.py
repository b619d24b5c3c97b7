"""The specialised FP32 FDM kernels (the order-3 plane-per-lane kernel and the
order-7 warp-per-element kernel) against the generic line-per-thread kernel on
the same level data (option fdmKernel = generic): bit-identical, RAS and ASM,
element counts that leave the last warp (five elements) or CTA (twenty)
partly filled."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pair(torch, N, n, schwarz, sched, level, eps=0.3):
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    base = (f"solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+{schwarz};maxIterations=200;"
            f"pMGSchedule={sched};coarseSolver=jpcg;coarseTol=1e-4;mgPrecision=mixed")
    fast = G.Elliptic(N, VX, EToV, EToB, base)
    gen = G.Elliptic(N, VX, EToV, EToB, base + ";fdmKernel=generic")
    m = fast.mg_level_size(level)
    u = torch.from_numpy(np.random.default_rng(n + 3 * level).uniform(-1, 1, m).astype(np.float32)).cuda()
    a, b = torch.full_like(u, float("nan")), torch.full_like(u, float("nan"))
    fast.mg_fdm(level, u, a)
    gen.mg_fdm(level, u, b)
    torch.cuda.synchronize()
    return a.cpu().numpy(), b.cpu().numpy()


@pytest.mark.parametrize("schwarz", ["ras", "asm"])
@pytest.mark.parametrize("n", [1, 2, 3, 7])
def test_order3_fdm_bit_identical(product_lib, torch_cuda, schwarz, n):
    """Order 3 as the fine level (E = 1, 8, 27, 343)."""
    a, b = _pair(torch_cuda, 3, n, schwarz, "p=3+degree=2,p=1,p=3+degree=2", 0)
    assert np.isfinite(b).all()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("schwarz", ["ras", "asm"])
def test_order3_fdm_bit_identical_mg_level(product_lib, torch_cuda, schwarz):
    """Order 3 as the middle level of the 7/3/1 schedule (E = 6^3)."""
    a, b = _pair(torch_cuda, 7, 6, schwarz, "p=7+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=7+degree=2", 1)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("schwarz", ["ras", "asm"])
def test_order7_fdm_matches_generic(product_lib, torch_cuda, schwarz):
    """The order-7 kernel against the generic one: the same sums in the same order, bit-identical."""
    a, b = _pair(torch_cuda, 7, 3, schwarz, "p=7+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=7+degree=2", 0)
    assert np.isfinite(b).all()
    assert np.array_equal(a, b)
