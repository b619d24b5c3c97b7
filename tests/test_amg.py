"""Algebraic multigrid coarse solve (coarseSolver = amg, nrsg_amg_*): the
library's host setup against the oracle's numpy restatement of the published
algorithms (oracle/amg_ref.py) on the assembled order-1 Kershaw operator —
same levels, same C/F splitting, interpolation and Galerkin operators to
rounding — and the restated cycle's convergence.  No GPU: the hierarchy is
built on the host."""
import numpy as np
import pytest
import scipy.sparse as sp

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import amg_ref as R
from oracle import oracle as O


def coarse_operator(n, eps=0.3, dirichlet=True):
    VX, EToV, EToB = W.kershaw_box(n, eps=eps, all_dirichlet=dirichlet)
    orc = O.Elliptic(1, VX, EToV, EToB, "preconditioner=jacobi")
    rp, cols, vals = G.host_assemble_operator(1, EToV, EToB, orc.get("ggeo"))[:3]
    return rp, cols, vals


def product_levels(amg):
    out = []
    for l in range(amg.num_levels):
        rp, ci, va, shape, lmax = amg.level_matrix(l, 0)
        A = sp.csr_matrix((va, ci, rp), shape=shape)
        P = None
        if l < amg.num_levels - 1:
            prp, pci, pva, pshape, _ = amg.level_matrix(l, 1)
            P = sp.csr_matrix((pva, pci, prp), shape=pshape)
        out.append((A, P, lmax if P is not None else None))
    return out


@pytest.mark.parametrize("n", [6, 10])
def test_amg_setup_matches_restatement(product_lib, n):
    rp, cols, vals = coarse_operator(n)
    A = sp.csr_matrix((vals, cols, rp), shape=(len(rp) - 1,) * 2)
    amg = G.Amg(rp, cols, vals)
    mine = product_levels(amg)
    ref = R.setup(A)
    assert [m[0].shape[0] for m in mine] == [r[0].shape[0] for r in ref]
    for (Am, Pm, lm), (Ar, Pr, lr) in zip(mine, ref):
        Am.sort_indices(), Ar.sort_indices()
        assert np.array_equal(Am.indptr, Ar.indptr) and np.array_equal(Am.indices, Ar.indices)
        assert np.abs(Am.data - Ar.data).max() <= 1e-12 * np.abs(Ar.data).max()
        if Pm is None:
            assert Pr is None
            continue
        Pm, Pr = sp.csr_matrix(Pm), sp.csr_matrix(Pr)
        Pm.sort_indices(), Pr.sort_indices()
        assert np.array_equal(Pm.indptr, Pr.indptr) and np.array_equal(Pm.indices, Pr.indices)
        assert np.abs(Pm.data - Pr.data).max() <= 1e-12
        # 60 power-iteration Rayleigh quotients against a converged Lanczos solve: within 2% (from below, so the
        # smoother weight 2 / (1.3 lmax) stays inside the interval where the sweep contracts)
        assert lr * 0.98 <= lm <= lr * (1 + 1e-9)
        # at most 4 weights per row; C points injected
        assert np.diff(Pm.indptr).max() <= 4
    # Galerkin: every coarse operator is R A P of the level above
    for (A0, P0, _), (A1, _, _) in zip(mine[:-1], mine[1:]):
        assert np.abs((P0.T @ A0 @ P0 - A1).toarray()).max() <= 1e-12 * np.abs(A1.data).max()


def test_amg_cycle_convergence(product_lib):
    rp, cols, vals = coarse_operator(12)
    A = sp.csr_matrix((vals, cols, rp), shape=(len(rp) - 1,) * 2)
    levels = R.setup(A)
    b = np.random.default_rng(1).standard_normal(A.shape[0])
    x = np.zeros_like(b)
    res = [np.linalg.norm(b)]
    for _ in range(8):
        x = x + R.vcycle(levels, b - A @ x)
        res.append(np.linalg.norm(b - A @ x))
    factor = (res[-1] / res[2]) ** (1 / 6)
    print(f"V-cycle convergence factor (Kershaw 12^3 order-1 operator): {factor:.3f}, levels "
          f"{[l[0].shape[0] for l in levels]}")
    assert factor < 0.6


def test_amg_rejects_bad_input(product_lib):
    with pytest.raises(G.NrsgError):
        G.Amg(np.array([0], dtype=np.int64), np.zeros(0, dtype=np.int64), np.zeros(0))
