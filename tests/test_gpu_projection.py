"""Solution projection on the GPU (initialGuess = projectionAconj / projection,
ellipticSolutionProjection.cpp) against the CPU oracle over a sequence of solves
that share one handle: the basis, its A-orthonormalisation and the projected
initial guess carry from solve to solve, so every solve of the sequence must
agree."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("form,nvec,precon", [("projectionAconj", 4, "jacobi"), ("projection", 4, "jacobi"),
                                              ("projectionAconj", 2, "jacobi"), ("projectionAconj", 3, "multigrid")])
def test_projection_sequence_parity(product_lib, oracle_mod, torch_cuda, form, nvec, precon):
    torch = torch_cuda
    N, n = 5, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    if precon == "jacobi":
        base = "preconditioner=jacobi;solver=pcg;residualTol=1e-10;maxIterations=3000"
    else:
        base = ("solver=pfcg;residualTol=1e-10;maxIterations=300;preconditioner=multigrid;"
                "smootherType=fourthoptcheby+asm;pMGSchedule=p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=5+degree=2;"
                "mgPrecision=fp64")
    opts = base + f";initialGuess={form};residualProjectionVectors={nvec};residualProjectionStart=2"
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    plain = G.Elliptic(N, VX, EToV, EToB, base)
    b1 = W.box_rhs(N, n, n, n, 21, orc.get("ggeo"))
    b2 = W.box_rhs(N, n, n, n, 22, orc.get("ggeo"))
    its_g, its_o, its_plain = [], [], []
    for k in range(7):
        rhs = np.cos(0.4 * k) * b1 + np.sin(0.4 * k) * b2
        xo, io = orc.solve(rhs)
        r = torch.from_numpy(rhs.copy()).cuda()
        x = torch.zeros_like(r)
        ig = el.solve(r, x)
        rp, xp = torch.from_numpy(rhs.copy()).cuda(), torch.zeros_like(r)
        ip = plain.solve(rp, xp)
        its_plain.append(ip["iterations"])
        torch.cuda.synchronize()
        assert ig["status"] == 0 and io["status"] == 0
        # the residual after projection is the small difference of two large vectors: compare it on
        # the scale of the unprojected residual, where both sides' rounding lives
        assert abs(ig["res0"] - io["res0"]) <= 1e-8 * ip["res0"], k
        assert abs(ig["iterations"] - io["iterations"]) <= 1, (k, ig["iterations"], io["iterations"])
        assert rel(x.cpu().numpy(), xo) < 1e-8, k
        its_g.append(ig["iterations"])
        its_o.append(io["iterations"])
    m, step = el.get("proj.vectors")
    assert step == 7 and 1 <= m <= nvec
    # the projected guess pays off once the basis spans the right-hand sides
    assert min(its_g[3:]) < min(its_plain) // 3, (its_g, its_plain)


def test_projection_off_leaves_solves_unchanged(product_lib, torch_cuda):
    torch = torch_cuda
    N, n = 3, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    base = "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=3000"
    a = G.Elliptic(N, VX, EToV, EToB, base)
    b = G.Elliptic(N, VX, EToV, EToB, base + ";initialGuess=previous")
    rhs = torch.from_numpy(W.box_rhs(N, n, n, n, 5, a.get("ggeo"))).cuda()
    xa, xb = torch.zeros_like(rhs), torch.zeros_like(rhs)
    ia, ib = a.solve(rhs.clone(), xa), b.solve(rhs.clone(), xb)
    assert ia["iterations"] == ib["iterations"]
    assert torch.equal(xa, xb)
