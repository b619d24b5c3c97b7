"""SEMFEM preconditioner (preconditioner = semfem, SEMFEMSolver.cpp): the
linear-tetrahedra operator on the fine level's GLL nodes (the same assembly as
the SEMFEM coarse discretization, pinned against the oracle on the CPU),
solved by one algebraic-multigrid V-cycle in FP32 per application.  Solves
converge to the oracle's FP64 Jacobi-PCG solution of the same problem, in far
fewer iterations than Jacobi."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,n", [(5, 4), (7, 4)])
@pytest.mark.parametrize("solver", ["pcg", "pfcg"])
def test_semfem_preconditioned_solve(product_lib, oracle_mod, torch_cuda, N, n, solver):
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    orc = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi;solver=pcg;residualTol=1e-12+relative;"
                     "maxIterations=20000")
    rhs = W.box_rhs(N, n, n, n, 17, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    its = {}
    for pre in ("semfem", "jacobi"):
        el = G.Elliptic(N, VX, EToV, EToB, f"preconditioner={pre};solver={solver};residualTol=1e-10+relative;"
                        "maxIterations=5000")
        r = torch.from_numpy(rhs.copy()).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        torch.cuda.synchronize()
        assert info["status"] == 0
        its[pre] = info["iterations"]
        if pre == "semfem":
            xg = x.cpu().numpy()
            err = float(np.linalg.norm(xg - xo) / np.linalg.norm(xo))
            lv = el.get("semfemLevels")
            print(f"N={N} E={n}^3 {solver}: SEMFEM {info['iterations']} iterations, AMG rows per level "
                  f"{lv[0::2].astype(int).tolist()}; error vs oracle {err:.2e}")
            assert err < 1e-8
    print(f"  Jacobi {its['jacobi']} iterations")
    assert its["semfem"] < its["jacobi"] / 3


def test_semfem_rejections(product_lib, torch_cuda):
    VX, EToV, EToB = W.kershaw_box(3, eps=0.3, all_dirichlet=False)
    with pytest.raises(G.NrsgError):
        G.Elliptic(3, VX, EToV, EToB, "preconditioner=semfem")  # all-Neumann
    VX, EToV, EToB = W.kershaw_box(3, eps=0.3)
    with pytest.raises(G.NrsgError):
        G.Elliptic(3, VX, EToV, EToB, "preconditioner=semfem;solver=pcg;nFields=3")
