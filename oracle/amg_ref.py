"""ORACLE — test infrastructure only: the product never imports this module.

Classical algebraic multigrid restated in numpy / scipy for the parity tests of
the library's coarse solve `coarseSolver = amg` (nrsg_amg_* in the C ABI).

The reference hands its assembled coarse operator to BoomerAMG (hypre 2.28.0,
a third-party library the reference vendors); the call site is
src/solvers/elliptic/MG/coarseLevel.cpp:77-133 with the settings of lines
79-92 (coarsening 10 = HMIS, interpolation 6 = extended+i, strength 0.25, one
V-cycle, Chebyshev smoothing of order 1) and hypreWrapper.cpp:120-200.  hypre
itself is not built or run here, so this restatement follows the published
algorithms, not hypre's code, and parity with BoomerAMG is unpinned; what is
pinned is the library's setup and V-cycle against this restatement:

* strength: j strongly influences i if -a_ij >= theta max_{k != i} (-a_ik);
* coarsening: the first pass of Ruge-Stueben (HMIS on one process), the
  unassigned point influencing the most unassigned points first, lowest index
  on ties;
* interpolation: extended+i (De Sterck, Falgout, Nolting, Yang, Numer. Linear
  Algebra Appl. 15 (2008) 115-139), truncated to the 4 largest weights per row
  with the row sum kept;
* Galerkin coarse operators R A P with R = P^T;
* smoothing: Chebyshev of degree 1 on D^-1 A over [0.3 lmax, lmax], i.e.
  x += 2 / (1.3 lmax) D^-1 r, one sweep down and one up; coarsest level solved
  exactly.
"""
import heapq

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _rows(A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    return A


def strength(A, theta=0.25):
    A = _rows(A)
    n = A.shape[0]
    indptr = [0]
    idx = []
    for i in range(n):
        c = A.indices[A.indptr[i]:A.indptr[i + 1]]
        v = A.data[A.indptr[i]:A.indptr[i + 1]]
        off = c != i
        if off.any():
            m = (-v[off]).max()
            if m > 0:
                idx += [int(j) for j, vv in zip(c, v) if j != i and -vv >= theta * m]
        indptr.append(len(idx))
    return sp.csr_matrix((np.ones(len(idx)), np.array(idx, dtype=np.int64), np.array(indptr)), shape=(n, n))


def rs_first_pass(S):
    n = S.shape[0]
    ST = sp.csr_matrix(S.T)
    ST.sort_indices()
    lam = np.diff(ST.indptr).astype(np.int64)
    state = np.zeros(n, np.int8)
    heap = [(-int(lam[i]), i) for i in range(n)]
    heapq.heapify(heap)
    while heap:
        l, i = heapq.heappop(heap)
        if state[i] != 0 or -l != lam[i]:
            continue
        if lam[i] == 0 and S.indptr[i + 1] == S.indptr[i]:
            state[i] = -1
            continue
        state[i] = 1
        for j in ST.indices[ST.indptr[i]:ST.indptr[i + 1]]:
            if state[j] == 0:
                state[j] = -1
                for k in S.indices[S.indptr[j]:S.indptr[j + 1]]:
                    if state[k] == 0:
                        lam[k] += 1
                        heapq.heappush(heap, (-int(lam[k]), int(k)))
        for k in S.indices[S.indptr[i]:S.indptr[i + 1]]:
            if state[k] == 0:
                lam[k] -= 1
                heapq.heappush(heap, (-int(lam[k]), int(k)))
    state[state == 0] = -1
    return state == 1


def ext_i_interp(A, S, isC, pmax=4):
    A = _rows(A)
    n = A.shape[0]
    cidx = -np.ones(n, np.int64)
    cidx[isC] = np.arange(int(isC.sum()))

    def row(i):
        return dict(zip(A.indices[A.indptr[i]:A.indptr[i + 1]].tolist(), A.data[A.indptr[i]:A.indptr[i + 1]].tolist()))

    rows, cols, vals = [], [], []
    for i in range(n):
        if isC[i]:
            rows.append(i), cols.append(cidx[i]), vals.append(1.0)
            continue
        Si = S.indices[S.indptr[i]:S.indptr[i + 1]].tolist()
        Ct = [j for j in Si if isC[j]]
        Fs = [j for j in Si if not isC[j]]
        seen = set(Ct)
        for k in Fs:
            for j in S.indices[S.indptr[k]:S.indptr[k + 1]].tolist():
                if isC[j] and j not in seen:
                    seen.add(j)
                    Ct.append(j)
        Ct.sort()
        if not Ct:
            continue
        ai = row(i)
        at = ai[i]
        w = {j: ai.get(j, 0.0) for j in Ct}
        Fset = set(Fs)
        for j, v in ai.items():
            if j == i or j in seen or j in Fset:
                continue
            at += v
        for k in Fs:
            ak = row(k)
            akk = ak[k]

            def bar(v):
                return v if (v < 0) != (akk < 0) and v != 0 else 0.0

            den = 0.0
            for l in Ct:
                den += bar(ak.get(l, 0.0))
            den += bar(ak.get(i, 0.0))
            aik = ai.get(k, 0.0)
            if den == 0:
                at += aik
                continue
            for j in Ct:
                w[j] += aik * bar(ak.get(j, 0.0)) / den
            at += aik * bar(ak.get(i, 0.0)) / den
        r = [(j, -w[j] / at) for j in Ct]
        if pmax > 0 and len(r) > pmax:
            tot = sum(x for _, x in r)
            order = sorted(range(len(r)), key=lambda q: -abs(r[q][1]))  # stable
            kept = [r[q] for q in order[:pmax]]
            ks = sum(x for _, x in kept)
            sc = tot / ks if ks != 0 else 1.0
            r = sorted((j, x * sc) for j, x in kept)
        for j, x in r:
            rows.append(i), cols.append(cidx[j]), vals.append(x)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, int(isC.sum())))


def setup(A, theta=0.25, pmax=4, max_coarse=50, max_levels=25):
    """Hierarchy [(A_l, P_l, lmax_l)] ending with (A_coarsest, None, None)."""
    A = _rows(A)
    levels = []
    while A.shape[0] > max_coarse and len(levels) < max_levels:
        S = strength(A, theta)
        isC = rs_first_pass(S)
        nc = int(isC.sum())
        if nc == 0 or nc == A.shape[0]:
            break
        P = ext_i_interp(A, S, isC, pmax)
        dinv = 1.0 / A.diagonal()
        s = np.sqrt(dinv)
        lmax = spla.eigsh(sp.diags(s) @ A @ sp.diags(s), k=1, which="LA", return_eigenvectors=False, tol=1e-8)[0]
        levels.append((A, P, float(lmax)))
        Ac = _rows(P.T @ A @ P)
        Ac.eliminate_zeros()
        A = Ac
    levels.append((A, None, None))
    return levels


def vcycle(levels, b, l=0):
    """One V-cycle from x = 0."""
    A, P, lmax = levels[l]
    if P is None:
        return np.linalg.solve(A.toarray(), b)
    wd = (2.0 / (1.3 * lmax)) / A.diagonal()
    x = wd * b
    r = b - A @ x
    x = x + P @ vcycle(levels, P.T @ r, l + 1)
    return x + wd * (b - A @ x)
