"""Kernel parity on the GPU: each CUDA kernel against the CPU oracle (and the
golden fixtures made from the reference's serial kernels).  The FP64 kernels of
the plain solve path (axhelm with stored geometry, geometric factors, the
Jacobi diagonal, gather-scatter, the fused PCG update and every weighted inner
product) are bit-identical to the oracle, which performs the same operations in
the same order; the reference-order oracle operator agrees to 1e-13 relative.
FP32 kernels: 1e-5."""
import os

import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz")


def dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6, 7, 8, 9])
@pytest.mark.parametrize("poisson", [True, False])
def test_ax_stored_f64(product_lib, oracle_mod, torch_cuda, N, poisson):
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(3, 2, 2, eps=0.3)
    l0, l1 = (1.0, 0.0) if poisson else (1.3, 0.7)
    el = O.Elliptic(N, VX, EToV, EToB, f"preconditioner=jacobi;poisson={int(poisson)};lambda0={l0};lambda1={l1}")
    q = np.random.default_rng(N).uniform(-1, 1, el.Nlocal)
    ref = el.ax(q)
    g, D = dev(torch, el.get("ggeo")), dev(torch, el.get("D"))
    qd = dev(torch, q)
    out = torch.zeros_like(qd)
    G.ax_stored_f64(N, el.E, g, D, l0, l1, poisson, qd, out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    assert relerr(out.cpu().numpy(), el.ax_ref(q)) < 1e-13


@pytest.mark.parametrize("N", [1, 3, 5, 7, 9])
def test_ax_stored_f32(product_lib, oracle_mod, torch_cuda, N):
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(2, 2, 3, eps=0.3)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    q = np.random.default_rng(N).uniform(-1, 1, el.Nlocal).astype(np.float32)
    ref = el.ax_fp32(q)
    g = dev(torch, el.get("ggeo"), torch.float32)
    D = dev(torch, el.get("D"), torch.float32)
    qd = dev(torch, q)
    out = torch.zeros_like(qd)
    G.ax_stored_f32(N, el.E, g, D, 1.0, 0.0, True, qd, out)
    torch.cuda.synchronize()
    assert relerr(out.cpu().numpy(), ref) < 1e-5


def test_ax_golden_reference(product_lib, torch_cuda):
    torch = torch_cuda
    g = np.load(GOLD)
    for N in (3, 7):
        E = g[f"N{N}_VX"].shape[0]
        gg, D, q = (dev(torch, g[f"N{N}_{k}"]) for k in ("ggeo", "D", "q"))
        out = torch.zeros_like(q)
        G.ax_stored_f64(N, E, gg, D, 1.0, 0.0, True, q, out)
        torch.cuda.synchronize()
        assert relerr(out.cpu().numpy(), g[f"N{N}_Aq_poisson"]) < 1e-13
        G.ax_stored_f64(N, E, gg, D, 1.3, 0.7, False, q, out)
        torch.cuda.synchronize()
        assert relerr(out.cpu().numpy(), g[f"N{N}_Aq_helmholtz"]) < 1e-13


@pytest.mark.parametrize("N", [1, 2, 4, 7, 9])
@pytest.mark.parametrize("helmholtz", [False, True])
def test_ax_trilinear_f64(product_lib, oracle_mod, torch_cuda, N, helmholtz):
    """Trilinear (recomputed geometry) axhelm: bit-identical to the oracle; lambda0 on the t-flux only, as the
    reference's kernel has it (ellipticPartialAxTrilinearHex3D.okl:154-157)."""
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(3, 3, 2, eps=0.7)
    l0, l1 = (1.3, 0.7) if helmholtz else (1.0, 0.0)
    el = O.Elliptic(N, VX, EToV, EToB, f"preconditioner=jacobi;elementMap=trilinear;poisson={int(not helmholtz)};"
                                       f"lambda0={l0};lambda1={l1}")
    q = np.random.default_rng(N + 10).uniform(-1, 1, el.Nlocal)
    ref = el.ax(q)
    z, w = O.gll(N)
    out = torch.zeros(el.Nlocal, dtype=torch.float64, device="cuda")
    G.ax_trilinear_f64(N, el.E, dev(torch, VX), dev(torch, z), dev(torch, w), dev(torch, el.get("D")), l0, l1,
                       not helmholtz, dev(torch, q), out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    if not helmholtz:
        # the recomputed geometry agrees with the stored-geometry operator
        ref2 = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi").ax(q)
        assert relerr(out.cpu().numpy(), ref2) < 1e-12


@pytest.mark.parametrize("N", [2, 5, 7])
def test_geometric_factors(product_lib, oracle_mod, torch_cuda, N):
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(3, 2, 2, eps=0.3)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    out = torch.zeros(7 * el.Nlocal, dtype=torch.float64, device="cuda")
    G.geometric_factors_f64(N, el.E, dev(torch, VX), out)
    assert np.array_equal(out.cpu().numpy(), el.get("ggeo"))


def test_gather_scatter_and_mask(product_lib, oracle_mod, torch_cuda):
    torch = torch_cuda
    N = 5
    VX, EToV, EToB = W.kershaw_box(3, eps=0.3)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    m = G.host_setup_maps(N, EToV, EToB)
    off, ids = m["gsOff"], m["gsIds"]
    q = np.random.default_rng(1).uniform(-1, 1, el.Nlocal)
    qd = dev(torch, q)
    G.gs_add_f64(len(off) - 1, dev(torch, off), dev(torch, ids), qd)
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), el.gs(q))  # same member order => bit-exact
    G.mask_f64(len(m["maskIds"]), dev(torch, m["maskIds"]), qd)
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), el.mask(el.gs(q)))


@pytest.mark.parametrize("z_bc", [1, 4])
def test_gather_scatter_large_groups(product_lib, oracle_mod, torch_cuda, z_bc):
    """The handle's gather-scatter (the plan kernel: pairs, groups of up to eight members from registers,
    larger groups member by member) on the twelve-sector fan mesh, whose axis groups have 12 and 24
    members: equal to the oracle's (same member order)."""
    torch = torch_cuda
    N = 4
    VX, EToV, EToB = W.axis_fan(12, 2, z_bc=z_bc)
    orc = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    el = G.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    q = np.random.default_rng(7).uniform(-1, 1, orc.Nlocal)
    qd = dev(torch, q)
    el.gs(qd)
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), orc.gs(q))


def test_fused_pcg_update_and_dot(product_lib, oracle_mod, torch_cuda):
    """r = fma(-alpha, Ap, r), x = fma(alpha, p, x) and (r, r)_w: bit-identical to the oracle; the
    weighted inner product is deterministic and bit-identical too."""
    torch = torch_cuda
    n = 1_000_003
    rng = np.random.default_rng(3)
    w, p, Ap, x, r = (rng.uniform(0.1, 1, n) for _ in range(5))
    alpha = 0.37
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    xd, rd = dev(torch, x), dev(torch, r)
    G.update_pcg_f64(n, dev(torch, w), dev(torch, p), dev(torch, Ap), alpha, xd, rd, out)
    torch.cuda.synchronize()
    xo, ro = x.copy(), r.copy()
    rr = O.update_pcg(w, p, Ap, alpha, xo, ro)
    assert np.array_equal(rd.cpu().numpy(), ro)
    assert np.array_equal(xd.cpu().numpy(), xo)
    assert out.item() == rr
    G.weighted_inner_prod_f64(n, dev(torch, w), dev(torch, p), dev(torch, Ap), out)
    torch.cuda.synchronize()
    v1 = out.item()
    G.weighted_inner_prod_f64(n, dev(torch, w), dev(torch, p), dev(torch, Ap), out)
    torch.cuda.synchronize()
    assert out.item() == v1  # deterministic
    assert v1 == O.wdot(w, p, Ap)


# sizes across the reduction's structure: one partial chunk, whole chunks, one group, the
# 4096-run limit (4096 x 1024 entries) and runs of several groups
@pytest.mark.parametrize("n", [1, 255, 256, 257, 1024, 1025, 70_001, 4096 * 1024 - 1, 4096 * 1024 + 1,
                               13_000_017])
def test_weighted_inner_prod_bitexact(product_lib, oracle_mod, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(n)
    w, a, b = rng.uniform(0, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    G.weighted_inner_prod_f64(n, dev(torch, w), dev(torch, a), dev(torch, b), out)
    torch.cuda.synchronize()
    assert out.item() == O.wdot(w, a, b)


@pytest.mark.parametrize("N", [1, 3, 5, 7, 9])
@pytest.mark.parametrize("poisson", [True, False])
def test_ax_fp32x2_is_fp64_accurate(product_lib, oracle_mod, torch_cuda, N, poisson):
    """FP32-pair axhelm against the FP64 oracle: within 2e-13 of max |Aq| (FP64 kernel: 1e-13)."""
    torch = torch_cuda
    VX, EToV, EToB = W.kershaw_box(3, 2, 2, eps=0.3)
    l0, l1 = (1.0, 0.0) if poisson else (1.3, 0.7)
    el = O.Elliptic(N, VX, EToV, EToB, f"preconditioner=jacobi;poisson={int(poisson)};lambda0={l0};lambda1={l1}")
    q = np.random.default_rng(N + 100).uniform(-1, 1, el.Nlocal)
    ref = el.ax(q)
    g = dev(torch, el.get("ggeo"))
    D = dev(torch, el.get("D"))
    gp = torch.zeros(2 * g.numel(), dtype=torch.float32, device="cuda")
    Dp = torch.zeros(2 * D.numel(), dtype=torch.float32, device="cuda")
    G.split_pairs(g.numel(), g, gp)
    G.split_pairs(D.numel(), D, Dp)
    out = torch.zeros(el.Nlocal, dtype=torch.float64, device="cuda")
    G.ax_fp32x2(N, el.E, gp, Dp, l0, l1, poisson, dev(torch, q), out)
    torch.cuda.synchronize()
    assert relerr(out.cpu().numpy(), ref) < 2e-13


@pytest.mark.parametrize("E", [1, 2, 3, 4, 7, 913, 5000])
@pytest.mark.parametrize("poisson", [True, False])
def test_ax_pipe_f32_bit_identical(product_lib, torch_cuda, E, poisson):
    """The bulk-copy pipelined FP32 order-7 axhelm equals the plain kernel bit for bit: partial last chunks
    (E not a multiple of 3), one chunk per CTA, and several chunks per CTA (both stage parities)."""
    torch = torch_cuda
    N, Np = 7, 512
    gen = torch.Generator(device="cuda").manual_seed(E + 17 * poisson)
    g = torch.rand(E * 7 * Np, device="cuda", generator=gen, dtype=torch.float32) + 0.5
    D = torch.from_numpy(O.dmatrix(N).astype(np.float32).ravel()).cuda()
    q = torch.rand(E * Np, device="cuda", generator=gen, dtype=torch.float32) - 0.5
    a_ref = torch.full_like(q, float("nan"))
    a_pipe = torch.full_like(q, float("nan"))
    cs = torch.cuda.current_stream().cuda_stream
    G.ax_stored_f32(N, E, g, D, 1.3, 0.7, poisson, q, a_ref, cs)
    G.ax_pipe_f32(N, E, g, D, 1.3, 0.7, poisson, q, a_pipe, cs)
    torch.cuda.synchronize()
    assert torch.equal(a_ref, a_pipe)


def test_ax_pipe_f32_rejects_unaligned_and_other_orders(product_lib, torch_cuda):
    torch = torch_cuda
    E, Np = 4, 512
    g = torch.rand(E * 7 * Np + 1, device="cuda")
    q = torch.rand(E * Np + 1, device="cuda")
    a = torch.empty(E * Np, device="cuda")
    D = torch.rand(64, device="cuda")
    cs = torch.cuda.current_stream().cuda_stream
    with pytest.raises(G.NrsgError):
        G.ax_pipe_f32(7, E, g[1:], D, 1.0, 0.0, True, q[:-1], a, cs)
    with pytest.raises(G.NrsgError):
        G.ax_pipe_f32(5, E, g[:-1], D, 1.0, 0.0, True, q[:-1], a, cs)


@pytest.mark.parametrize("variant", ["axPipeline=1", "axConst=1"])
def test_mg_solve_same_with_and_without_ax_pipeline(product_lib, torch_cuda, variant):
    torch = torch_cuda
    N, n = 7, 5
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = ("solver=pfcg;residualTol=1e-8+relative;maxIterations=200;preconditioner=multigrid;"
            "smootherType=fourthoptcheby+ras;pMGSchedule=p=7+degree=5,p=3+degree=5,p=1,p=3+degree=5,p=7+degree=5;"
            "mgPrecision=mixed")
    a = G.Elliptic(N, VX, EToV, EToB, opts + ";" + variant)
    b = G.Elliptic(N, VX, EToV, EToB, opts)
    rhs = torch.from_numpy(W.box_rhs(N, n, n, n, 3, a.get("ggeo"))).cuda()
    xa, xb = torch.zeros_like(rhs), torch.zeros_like(rhs)
    ia, ib = a.solve(rhs.clone(), xa), b.solve(rhs.clone(), xb)
    assert ia["status"] == 0 and ia["iterations"] == ib["iterations"]
    assert torch.equal(xa, xb)


@pytest.mark.parametrize("E", [1, 2, 7, 1000, 2433])
@pytest.mark.parametrize("poisson", [True, False])
@pytest.mark.parametrize("prefetch", [False, True])
def test_ax_const_f32_bit_identical(product_lib, torch_cuda, E, poisson, prefetch):
    """The FP32 order-7 axhelm with D in constant memory and registers equals the default kernel bit for bit
    (same operands, same operation order); so does its persistent form that prefetches each CTA's next
    element pair into L2 (E = 2433: more pairs than resident CTAs, an odd last pair)."""
    torch = torch_cuda
    N, Np = 7, 512
    gen = torch.Generator(device="cuda").manual_seed(3 * E + poisson)
    g = torch.rand(E * 7 * Np, device="cuda", generator=gen, dtype=torch.float32) + 0.5
    D = torch.from_numpy(O.dmatrix(N).astype(np.float32).ravel()).cuda()
    q = torch.rand(E * Np, device="cuda", generator=gen, dtype=torch.float32) - 0.5
    a_ref = torch.full_like(q, float("nan"))
    a_c = torch.full_like(q, float("nan"))
    cs = torch.cuda.current_stream().cuda_stream
    G.ax_stored_f32(N, E, g, D, 1.3, 0.7, poisson, q, a_ref, cs)
    (G.ax_const_prefetch_f32 if prefetch else G.ax_const_f32)(N, E, g, D, 1.3, 0.7, poisson, q, a_c, cs)
    torch.cuda.synchronize()
    assert torch.equal(a_ref, a_c)


def test_ax_const_prefetch_unaligned_pointers(product_lib, torch_cuda):
    """The persistent prefetching axhelm with q and the geometric factors 4 bytes off a 16-byte boundary (the
    bulk L2 prefetch needs 16-byte alignment, so it is skipped): still bit-identical to the default kernel."""
    torch = torch_cuda
    N, Np, E = 7, 512, 1500
    gen = torch.Generator(device="cuda").manual_seed(41)
    gbuf = torch.rand(E * 7 * Np + 1, device="cuda", generator=gen, dtype=torch.float32) + 0.5
    qbuf = torch.rand(E * Np + 1, device="cuda", generator=gen, dtype=torch.float32) - 0.5
    g, q = gbuf[1:], qbuf[1:]
    assert g.data_ptr() % 16 == 4 and q.data_ptr() % 16 == 4
    D = torch.from_numpy(O.dmatrix(N).astype(np.float32).ravel()).cuda()
    a_ref = torch.full((E * Np,), float("nan"), device="cuda")
    a_pf = torch.full_like(a_ref, float("nan"))
    cs = torch.cuda.current_stream().cuda_stream
    G.ax_stored_f32(N, E, g, D, 1.0, 0.0, True, q, a_ref, cs)
    G.ax_const_prefetch_f32(N, E, g, D, 1.0, 0.0, True, q, a_pf, cs)
    torch.cuda.synchronize()
    assert torch.equal(a_ref, a_pf)
