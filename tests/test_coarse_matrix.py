"""Assembled level operator (the coarse-solver matrix), host code of the library
against the oracle's restatement of the reference's FEM matrix builder and
against the oracle's element-wise operator.  No GPU."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

sp = pytest.importorskip("scipy.sparse")


def _dense(rp, cols, vals):
    n = len(rp) - 1
    return sp.csr_matrix((vals, cols, rp), shape=(n, n))


def _check(N, VX, EToV, EToB, lam0=1.0, lam1=0.0, poisson=True):
    opts = "preconditioner=jacobi" + ("" if poisson else f";poisson=0;lambda0={lam0!r};lambda1={lam1!r}")
    orc = O.Elliptic(N, VX, EToV, EToB, opts)
    gg = orc.get("ggeo")
    rp, cols, vals, rown = G.host_assemble_operator(N, EToV, EToB, gg, lam0, lam1, poisson)
    rp2, cols2, vals2 = orc.assemble(lam0, lam1, poisson)
    # same sparsity (exact zeros dropped in both), same values up to summation order
    assert np.array_equal(rp, rp2) and np.array_equal(cols, cols2)
    assert np.max(np.abs(vals - vals2)) <= 1e-14 * np.max(np.abs(vals2))
    # rows are the masked gather groups, in order
    off, ids = orc.get("gsOff"), orc.get("gsIds")
    assert len(rp) - 1 == len(off) - 1
    for g in (0, len(off) // 2, len(off) - 2):
        assert np.all(rown[ids[off[g]:off[g + 1]]] == g)
    assert np.all(rown[orc.get("maskIds")] == -1)
    # the matrix is the level operator on continuous, masked vectors
    A = _dense(rp, cols, vals)
    u = np.random.default_rng(3).standard_normal(A.shape[0])
    uE = np.where(rown >= 0, u[np.maximum(rown, 0)], 0.0)
    AuE = orc.operator(uE)
    ref = np.zeros(A.shape[0])
    m = rown >= 0
    ref[rown[m]] = AuE[m]
    assert np.max(np.abs(A @ u - ref)) <= 1e-13 * np.max(np.abs(ref))
    # symmetric
    assert abs(A - A.T).max() <= 1e-15 * abs(A).max()
    return A


@pytest.mark.parametrize("N,n,eps", [(1, 4, 0.3), (1, 6, 0.3), (1, 3, 1.0), (2, 2, 0.3), (3, 2, 0.3)])
def test_assembled_operator_matches_oracle(product_lib, oracle_mod, N, n, eps):
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    A = _check(N, VX, EToV, EToB)
    widths = np.diff(A.indptr)
    if N == 1:
        assert widths.max() <= 27
    if N == 1 and eps == 1.0:
        # rectilinear elements: the cross terms vanish exactly, a 7-point stencil remains
        assert widths.max() == 7


def test_assembled_helmholtz_operator(product_lib, oracle_mod):
    VX, EToV, EToB = W.kershaw_box(4, eps=0.3)
    _check(1, VX, EToV, EToB, lam0=1.3, lam1=0.7, poisson=False)


def test_assembled_operator_neumann_faces(product_lib, oracle_mod):
    VX, EToV, EToB = W.kershaw_box(3, 2, 2, eps=0.3, all_dirichlet=False)
    EToB = EToB.copy()
    EToB[0, 4] = 1
    _check(1, VX, EToV, EToB)


@pytest.mark.parametrize("N,n,eps,poisson", [(3, 3, 0.3, True), (7, 2, 1.0, True), (5, 3, 0.5, False)])
def test_galerkin_operator_matches_oracle(product_lib, oracle_mod, N, n, eps, poisson):
    """coarseGridDiscretization = FEM+Galerkin: the library's B^T A_f B (host code) equals the oracle's
    restatement of ellipticBuildFEMGalerkinHex3D bit for bit; rows are the order-1 level's masked groups."""
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    fine = O.Elliptic(N, VX, EToV, EToB, "preconditioner=none")
    coarse = O.Elliptic(1, VX, EToV, EToB, "preconditioner=none")
    l1 = 0.0 if poisson else 2.0
    ref = fine.assemble_galerkin(coarse, 1.0, l1, poisson)
    rp, cols, vals, ron = G.host_assemble_galerkin(N, EToV, EToB, fine.get("ggeo"), 1.0, l1, poisson)
    assert np.array_equal(rp, ref[0]) and np.array_equal(cols, ref[1]) and np.array_equal(vals, ref[2])
    fem = G.host_assemble_operator(1, EToV, EToB, coarse.get("ggeo"))
    assert np.array_equal(ron, fem[3])
    A = sp.csr_matrix((vals, cols, rp))
    # symmetric up to the FP32 rounding of the fine operator; positive diagonal
    assert abs(A - A.T).max() <= 1e-6 * abs(A).max()
    assert (A.diagonal() > 0).all()


def test_galerkin_of_an_order_one_level_is_its_fem_operator(product_lib, oracle_mod):
    """With an order-1 fine level the coarse basis is the identity: B^T A B is the FEM operator evaluated in
    FP32 (the pfloat ellipticAx the reference projects)."""
    VX, EToV, EToB = W.kershaw_box(4, eps=0.3)
    c = O.Elliptic(1, VX, EToV, EToB, "preconditioner=none")
    rp, cols, vals, _ = G.host_assemble_galerkin(1, EToV, EToB, c.get("ggeo"))
    frp, fcols, fvals, _ = G.host_assemble_operator(1, EToV, EToB, c.get("ggeo"))
    Ag, Af = sp.csr_matrix((vals, cols, rp)), sp.csr_matrix((fvals, fcols, frp))
    assert abs(Ag - Af).max() <= 1e-6 * abs(Af).max()


def test_oracle_mg_with_galerkin_coarse_converges(oracle_mod):
    VX, EToV, EToB = W.kershaw_box(4, eps=0.3)
    opts = ("solver=pfcg;residualTol=1e-8+relative;maxIterations=200;preconditioner=multigrid;"
            "smootherType=fourthoptcheby+asm;pMGSchedule=p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=5+degree=2;"
            "mgPrecision=fp64")
    its = {}
    for g in ("fem", "fem+galerkin"):
        el = O.Elliptic(5, VX, EToV, EToB, opts + f";coarseGridDiscretization={g}")
        x, info = el.solve(W.box_rhs(5, 4, 4, 4, 3, el.get("ggeo")))
        assert info["status"] == 0 and info["res"] <= 1e-8 * info["res0"]
        its[g] = info["iterations"]
    assert abs(its["fem"] - its["fem+galerkin"]) <= 3, its


@pytest.mark.parametrize("N,n,eps", [(1, 4, 0.3), (1, 3, 1.0), (3, 3, 0.5), (7, 2, 1.0)])
def test_semfem_operator_matches_oracle(product_lib, oracle_mod, N, n, eps):
    """coarseGridDiscretization = SEMFEM: the library's linear-tetrahedron operator on the GLL grid equals
    the oracle's restatement of SEMFEMSolver_t::build (FP32 accumulation in the reference's loop order) up to
    rounding residues of exact zeros (their node coordinates are interpolated by different code)."""
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    orc = O.Elliptic(N, VX, EToV, EToB, "preconditioner=none")
    rp, cols, vals = orc.assemble_semfem(1.3)
    prp, pcols, pvals, ron = G.host_assemble_semfem(N, VX, EToV, EToB, 1.3)
    A, P = sp.csr_matrix((vals, cols, rp)), sp.csr_matrix((pvals, pcols, prp))
    assert A.shape == P.shape
    assert abs(A - P).max() <= 1e-6 * abs(A).max()  # FP32 entries
    if N == 1:
        assert np.array_equal(rp, prp) and np.array_equal(cols, pcols) and np.array_equal(vals, pvals)
    # symmetric with a positive diagonal; without a mask the constants are in its kernel
    assert abs(A - A.T).max() <= 1e-6 * abs(A).max()
    assert (P.diagonal() > 0).all()
    assert ron.shape[0] == orc.Nlocal
    nrp, ncols, nvals, _ = G.host_assemble_semfem(N, VX, EToV, np.zeros_like(EToB), 1.3)
    Pn = sp.csr_matrix((nvals, ncols, nrp))
    assert np.abs(Pn @ np.ones(Pn.shape[0])).max() <= 1e-5 * abs(Pn).max()


def test_oracle_mg_with_semfem_coarse_converges(oracle_mod):
    VX, EToV, EToB = W.kershaw_box(4, eps=0.3)
    opts = ("solver=pfcg;residualTol=1e-8+relative;maxIterations=200;preconditioner=multigrid;"
            "smootherType=fourthoptcheby+asm;pMGSchedule=p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=5+degree=2;"
            "mgPrecision=fp64;coarseGridDiscretization=semfem")
    el = O.Elliptic(5, VX, EToV, EToB, opts)
    x, info = el.solve(W.box_rhs(5, 4, 4, 4, 3, el.get("ggeo")))
    assert info["status"] == 0 and info["res"] <= 1e-8 * info["res0"]
    assert info["iterations"] <= 15
