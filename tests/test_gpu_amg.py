"""Algebraic multigrid coarse solve on the GPU: the device V-cycle against the
oracle's numpy restatement applied to the library's own hierarchy (FP64, to
rounding), and p-multigrid solves with coarseSolver = amg (one V-cycle per
coarse solve, as the reference runs BoomerAMG) against the Jacobi-PCG coarse
solve and the FP64 oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import amg_ref as R
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SCHED7 = "p=7+degree=5,p=3+degree=5,p=1,p=3+degree=5,p=7+degree=5"


@pytest.mark.parametrize("n", [6, 16])
def test_amg_device_vcycle(product_lib, torch_cuda, n):
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    orc = O.Elliptic(1, VX, EToV, EToB, "preconditioner=jacobi")
    rp, cols, vals = G.host_assemble_operator(1, EToV, EToB, orc.get("ggeo"))[:3]
    amg = G.Amg(rp, cols, vals)
    levels = []
    for l in range(amg.num_levels):
        arp, aci, ava, shape, lmax = amg.level_matrix(l, 0)
        P = None
        if l < amg.num_levels - 1:
            prp, pci, pva, pshape, _ = amg.level_matrix(l, 1)
            P = sp.csr_matrix((pva, pci, prp), shape=pshape)
        levels.append((sp.csr_matrix((ava, aci, arp), shape=shape), P, lmax if P is not None else None))
    b = np.random.default_rng(n).standard_normal(amg.n)
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros_like(bd)
    amg.vcycle(bd, xd)
    want = R.vcycle(levels, b)
    err = np.abs(xd.cpu().numpy() - want).max() / np.abs(want).max()
    print(f"E={n}^3: device V-cycle vs restatement {err:.2e}, levels {[l[0].shape[0] for l in levels]}")
    assert err < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_mg_solve_with_amg_coarse(product_lib, oracle_mod, torch_cuda, prec):
    torch = torch_cuda
    n, N = 6, 7
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    base = (f"solver=pfcg;preconditioner=multigrid;smootherType=fourthoptcheby+ras;pMGSchedule={SCHED7};"
            f"residualTol=1e-8+relative;maxIterations=200;mgPrecision={prec}")
    orc = O.Elliptic(N, VX, EToV, EToB, base.replace("mgPrecision=mixed", "mgPrecision=fp64") +
                     ";coarseSolver=jpcg;coarseTol=1e-4")
    rhs = W.box_rhs(N, n, n, n, 3, orc.get("ggeo"))
    xo, io = orc.solve(rhs)
    its = {}
    for cs in ("jpcg;coarseTol=1e-4", "amg"):
        el = G.Elliptic(N, VX, EToV, EToB, base + f";coarseSolver={cs}")
        r = torch.from_numpy(rhs.copy()).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        torch.cuda.synchronize()
        assert info["status"] == 0 and info["res"] <= 1e-8 * info["res0"]
        its[cs] = info["iterations"]
        xg = x.cpu().numpy()
        if cs == "amg":
            lv = el.get("mg.amgLevels")
            err = float(np.linalg.norm(xg - xo) / np.linalg.norm(xo))
            print(f"{prec}: iterations jpcg {its['jpcg;coarseTol=1e-4']}, amg {its['amg']}, oracle {io['iterations']}; "
                  f"AMG rows per level {lv[0::2].astype(int).tolist()}; error vs FP64 oracle {err:.2e}")
            assert len(lv) >= 4 and lv[0] > lv[2]
            assert err < 1e-7
    assert its["amg"] <= its["jpcg;coarseTol=1e-4"] + 2


def test_amg_coarse_rejected_for_all_neumann(product_lib, torch_cuda):
    VX, EToV, EToB = W.kershaw_box(3, eps=0.3, all_dirichlet=False)
    with pytest.raises(G.NrsgError):
        G.Elliptic(3, VX, EToV, EToB, "preconditioner=multigrid;smootherType=cheby+asm;coarseSolver=amg;"
                   "pMGSchedule=p=3+degree=2,p=1,p=3+degree=2")


@pytest.mark.parametrize("n", [1, 7, 50])
def test_amg_dense_only(product_lib, torch_cuda, n):
    """Operators of at most 50 rows skip coarsening: the V-cycle is the dense coarsest solve alone (exact)."""
    torch = torch_cuda
    rng = np.random.default_rng(n)
    M = rng.standard_normal((n, n))
    A = sp.csr_matrix(M @ M.T + n * np.eye(n))
    amg = G.Amg(A.indptr.astype(np.int64), A.indices.astype(np.int64), A.data)
    assert amg.num_levels == 1
    b = rng.standard_normal(n)
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros_like(bd)
    amg.vcycle(bd, xd)
    want = np.linalg.solve(A.toarray(), b)
    assert np.abs(xd.cpu().numpy() - want).max() <= 1e-12 * np.abs(want).max()
