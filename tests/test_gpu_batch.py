"""Batched and resumable solves (nrsg_elliptic_solve_batch, solve_begin / solve_advance): independent
solves stepped together give exactly the results of solving them one by one."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SCHED = {3: "p=3+degree=2,p=1,p=3+degree=2", 5: "p=5+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=5+degree=2",
         7: "p=7+degree=4,p=3+degree=4,p=1,p=3+degree=4,p=7+degree=4"}


def problems():
    out = []
    for k, (N, n, eps, kind) in enumerate([(3, 6, 0.3, "mixed"), (5, 4, 0.7, "fp64"), (7, 3, 1.0, "jacobi"),
                                            (7, 4, 0.3, "mixed"), (5, 3, 0.5, "fp32")]):
        if kind == "jacobi":
            opts = "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=3000"
        else:
            opts = (f"solver=pfcg;residualTol=1e-8+relative;maxIterations=300;preconditioner=multigrid;"
                    f"smootherType=fourthoptcheby+asm;pMGSchedule={SCHED[N]};mgPrecision={kind}")
        VX, EToV, EToB = W.kershaw_box(n, eps=eps)
        out.append((N, n, VX, EToV, EToB, opts, 100 + k))
    return out


def setup_all(torch):
    els, rhs = [], []
    for N, n, VX, EToV, EToB, opts, seed in problems():
        el = G.Elliptic(N, VX, EToV, EToB, opts)
        els.append(el)
        rhs.append(torch.from_numpy(W.box_rhs(N, n, n, n, seed, el.get("ggeo"))).cuda())
    return els, rhs


def test_batch_matches_individual_solves(product_lib, torch_cuda):
    torch = torch_cuda
    els, rhs = setup_all(torch)
    ref = []
    for el, b in zip(els, rhs):
        r, x = b.clone(), torch.zeros_like(b)
        info = el.solve(r, x)
        ref.append((info, x.cpu().numpy()))
    rs = [b.clone() for b in rhs]
    xs = [torch.zeros_like(b) for b in rhs]
    infos = G.solve_batch(els, rs, xs)
    for (ri, rx), info, x in zip(ref, infos, xs):
        assert info["status"] == 0
        assert info["iterations"] == ri["iterations"]
        assert info["res"] == ri["res"]
        assert np.array_equal(x.cpu().numpy(), rx)


def test_resumable_solve_matches_blocking(product_lib, torch_cuda):
    torch = torch_cuda
    els, rhs = setup_all(torch)
    el, b = els[3], rhs[3]
    r, x = b.clone(), torch.zeros_like(b)
    ref = el.solve(r, x)
    xr = x.cpu().numpy()
    r2, x2 = b.clone(), torch.zeros_like(b)
    el.solve_begin(r2, x2)
    polls, info = 0, None
    while info is None:
        info = el.solve_advance()
        polls += 1
    assert info["iterations"] == ref["iterations"] and info["status"] == 0
    assert np.array_equal(x2.cpu().numpy(), xr)
    assert polls > info["iterations"]  # advance returned before the device had finished at least once per iteration
    # a finished handle keeps returning its result; a new solve can start on it
    assert el.solve_advance()["iterations"] == info["iterations"]
    r3, x3 = b.clone(), torch.zeros_like(b)
    el.solve_begin(r3, x3)
    while el.solve_advance() is None:
        pass
    assert np.array_equal(x3.cpu().numpy(), xr)


def test_batch_reports_iteration_limit(product_lib, torch_cuda):
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(3, eps=0.3)
    ok = G.Elliptic(5, VX, EToV, EToB, "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=3000")
    lim = G.Elliptic(5, VX, EToV, EToB, "preconditioner=jacobi;solver=pcg;residualTol=1e-12+relative;maxIterations=5")
    b = torch.from_numpy(W.box_rhs(5, 3, 3, 3, 7, ok.get("ggeo"))).cuda()
    infos = G.solve_batch([ok, lim], [b.clone(), b.clone()], [torch.zeros_like(b), torch.zeros_like(b)])
    assert infos[0]["status"] == 0 and infos[1]["status"] == 1 and infos[1]["iterations"] == 5


@pytest.mark.parametrize("budget", ["all", "one"])
def test_library_server_alone_vs_in_mix(product_lib, torch_cuda, budget):
    """The library's request scheduler (nrsg_server_*): requests on resident handles, several per handle, with
    tolerances 1e-6 / 1e-8 / 1e-10, stepped together one Krylov iteration at a time; every result is bit
    for bit the result of the same request solved alone.  With a budget below two handles' device
    footprint at most one request is in flight at any step."""
    torch = torch_cuda
    els, rhs = setup_all(torch)
    foot = [int(el.get("deviceBytes")[0]) for el in els]
    assert all(f > 0 for f in foot)
    tols = [1e-6, 1e-8, 1e-10]
    reqs = []  # (handle index, tolerance, seed scale)
    for k in range(9):
        reqs.append((k % len(els), tols[k % 3], 1.0 + 0.25 * k))
    # alone
    alone = []
    for h, tol, sc in reqs:
        el = els[h]
        el.set_tolerance(tol)
        r = rhs[h] * sc
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        alone.append((x.cpu().numpy(), info["iterations"]))
    # in the mix, through the library scheduler
    srv = G.Server(sum(foot) * 2 if budget == "all" else min(foot) + 1)
    bufs, ids = [], []
    for h, tol, sc in reqs:
        r = rhs[h] * sc
        x = torch.zeros_like(r)
        bufs.append((r, x))
        ids.append(srv.submit(els[h], r, x, tol))
    results, max_inflight = {}, 0
    for _ in range(200000):
        a, q = srv.step()
        max_inflight = max(max_inflight, a)
        for rid, info in srv.poll():
            results[rid] = info
        if a == 0 and q == 0:
            break
    for rid, info in srv.poll():
        results[rid] = info
    assert len(results) == len(reqs)
    if budget == "one":
        assert max_inflight == 1
    else:
        assert max_inflight >= 2
    torch.cuda.synchronize()
    for k, rid in enumerate(ids):
        assert results[rid]["status"] == 0
        assert results[rid]["iterations"] == alone[k][1]
        assert np.array_equal(bufs[k][1].cpu().numpy(), alone[k][0])
