"""A solve set up from a mesh read through the .re2 path (library reader +
parCon numbering) is bit-identical to the solve on the generator's mesh:
the vertex numbering only names vertices, so gather groups, masks, the
assembled coarse operator and every kernel see the same data."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import re2 as R
from nekrs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["mixed", "jacobi"])
def test_solve_on_re2_mesh_is_bit_identical(product_lib, torch_cuda, tmp_path, kind):
    torch = torch_cuda
    N, n = 7, 4
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    _, cbc = R.box(n, n, n, *(np.arange(n + 1.0),) * 3, ("O",) * 6)
    p = tmp_path / "k.re2"
    R.write_re2(p, VX, cbc)
    VX2, EToV2, EToB2 = R.mesh_from_re2(p, {"O": R.NRSG_BC_DIRICHLET})
    assert not np.array_equal(EToV, EToV2)
    if kind == "jacobi":
        opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=3000"
    else:
        opts = ("solver=pfcg;residualTol=1e-8+relative;maxIterations=200;preconditioner=multigrid;"
                "smootherType=fourthoptcheby+ras;pMGSchedule=p=7+degree=5,p=3+degree=5,p=1,p=3+degree=5,"
                "p=7+degree=5;mgPrecision=mixed")
    a = G.Elliptic(N, VX, EToV, EToB, opts)
    b = G.Elliptic(N, VX2, EToV2, EToB2, opts)
    rhs = torch.from_numpy(W.box_rhs(N, n, n, n, 9, a.get("ggeo"))).cuda()
    xa, xb = torch.zeros_like(rhs), torch.zeros_like(rhs)
    ia = a.solve(rhs.clone(), xa)
    ib = b.solve(rhs.clone(), xb)
    assert ia["status"] == 0 and ib["status"] == 0
    assert ia["iterations"] == ib["iterations"] and ia["res"] == ib["res"]
    assert torch.equal(xa, xb)
