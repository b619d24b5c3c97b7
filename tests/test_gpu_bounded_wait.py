"""The persistent coarse-level kernel's grid-barrier waits are bounded: every
wait gives up after a set number of polls, records an error flag and returns,
and the solve then reports NRSG_ERR_CUDA with the grid-barrier message instead
of hanging.  The test makes every wait run out by raising each barrier's
arrival target by one (option coarseBarrierExtra, a count nothing ever
reaches) under a small poll limit (coarseSpinLimit), on a one-CTA coarse level
and on a cooperative many-CTA one, and checks that the device context stays
usable: a solve without the knob on the same process succeeds afterwards."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SCHED3 = "p=3+degree=2,p=1,p=3+degree=2"


# coarse level of 27 rows (one CTA), 6859 rows (two CTAs: the cluster layout, launched cooperatively with the
# counting barrier under the test knob) and 42875 rows (many CTAs of a cooperative launch)
@pytest.mark.parametrize("n", [4, 20, 36])
def test_coarse_grid_barrier_wait_runs_out(product_lib, torch_cuda, n):
    torch = torch_cuda
    N = 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    base = ("solver=pfcg;preconditioner=multigrid;smootherType=cheby+asm;mgPrecision=fp64;"
            f"residualTol=1e-9+relative;maxIterations=20;pMGSchedule={SCHED3};coarsePersistent=1")
    el = G.Elliptic(N, VX, EToV, EToB, base + ";coarseSpinLimit=4096;coarseBarrierExtra=1")
    if n > 4:
        grid = el.get("mg.coarseMatrix")[3]
        assert grid >= (2 if n == 20 else 8)  # several CTAs, all waiting at every barrier
    rhs = W.box_rhs(N, n, n, n, 5, el.get("ggeo"))
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    with pytest.raises(G.NrsgError) as e:
        el.solve(r, x)
    assert e.value.code == 6  # NRSG_ERR_CUDA
    assert "grid barrier" in str(e.value)
    torch.cuda.synchronize()  # no sticky CUDA error: the kernels returned
    # the same problem without the knob, in the same process: solved
    ok = G.Elliptic(N, VX, EToV, EToB, base.replace("maxIterations=20", "maxIterations=200"))
    r2 = torch.from_numpy(rhs.copy()).cuda()
    x2 = torch.zeros_like(r2)
    info = ok.solve(r2, x2)
    assert info["status"] == 0
    assert ok.get("mg.coarseError")[0] == 0
    assert np.isfinite(x2.cpu().numpy()).all()
