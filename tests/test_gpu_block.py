"""Block (vector) Helmholtz on the GPU against the oracle's restatement: the
block axhelm with scalar and per-node coefficients, the stress (symmetric
gradient) operator, the block Jacobi diagonal, and whole PCG solves over 3
fields (the velocity solve next to the pressure solve)."""
import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BASE = "preconditioner=jacobi;solver=pcg+block;residualTol=1e-8+relative;maxIterations=3000;poisson=0;lambda0=1.0;lambda1=0.0"


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def coefficient_fields(el_o, nf):
    x, y, z = el_o.get("x"), el_o.get("y"), el_o.get("z")
    mu = 1.0 + 0.5 * np.sin(3 * x) * np.cos(2 * y) + 0.2 * z  # viscosity-like, positive
    h = 20.0 + 5.0 * np.cos(x + y + z)                         # rho * bd0 / dt-like
    return mu, h


@pytest.mark.parametrize("N,nf,stress,kind", [(3, 3, False, "scalar"), (5, 3, False, "shared"),
                                              (7, 2, False, "perfield"), (5, 3, True, "scalar"),
                                              (7, 3, True, "shared"), (4, 3, True, "perfield")])
def test_block_operator_and_jacobi(product_lib, oracle_mod, torch_cuda, N, nf, stress, kind):
    torch = torch_cuda
    n = 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = BASE.replace("pcg+block", "pcg") + f";nFields={nf};lambda1=0.8" + (";stressFormulation=true" if stress else "")
    orc = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    Nl = orc.get("invDegree").size
    lam0 = lam1 = None
    loff = 0
    if kind != "scalar":
        mu, h = coefficient_fields(orc, nf)
        if kind == "perfield":
            lam0 = np.concatenate([mu * (1 + 0.1 * f) for f in range(nf)])
            lam1 = np.concatenate([h * (1 - 0.1 * f) for f in range(nf)])
            loff = Nl
        else:
            lam0, lam1 = mu, h
        el.set_coefficients(torch.from_numpy(lam0).cuda(), torch.from_numpy(lam1).cuda(), loff)
    q = np.random.default_rng(N).standard_normal(nf * Nl)
    ref = orc.block_ax(q, nf=nf, stress=stress, poisson=False, lam0=lam0, lam1=lam1, l0=1.0, l1=0.8, loffset=loff)
    out = torch.zeros(nf * Nl, dtype=torch.float64, device="cuda")
    el.ax(torch.from_numpy(q).cuda(), out)
    torch.cuda.synchronize()
    assert rel(out.cpu().numpy(), ref) < 1e-13
    dref = orc.block_inv_diag(nf=nf, poisson=False, lam0=lam0, lam1=lam1, l0=1.0, l1=0.8, loffset=loff)
    assert rel(el.get("invDiag"), dref) < 1e-13


@pytest.mark.parametrize("N,stress,kind", [(5, False, "shared"), (7, True, "shared"), (5, True, "scalar"),
                                           (3, False, "perfield")])
def test_block_pcg_solve_parity(product_lib, oracle_mod, torch_cuda, N, stress, kind):
    torch = torch_cuda
    n = 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = BASE + ";lambda1=10.0;residualTol=1e-10+relative" + (";stressFormulation=true" if stress else "")
    orc = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    Nl = orc.get("invDegree").size
    lam0 = lam1 = None
    loff = 0
    if kind != "scalar":
        mu, h = coefficient_fields(orc, 3)
        if kind == "perfield":
            lam0, lam1, loff = np.concatenate([mu, 1.2 * mu, 0.8 * mu]), np.concatenate([h, h, 2 * h]), Nl
        else:
            lam0, lam1 = mu, h
        el.set_coefficients(torch.from_numpy(lam0).cuda(), torch.from_numpy(lam1).cuda(), loff)
    rhs = np.concatenate([W.box_rhs(N, n, n, n, s, orc.get("ggeo")) for s in (5, 6, 7)])
    xo, io = orc.block_solve(rhs, nf=3, stress=stress, poisson=False, lam0=lam0, lam1=lam1, l0=1.0, l1=10.0,
                             loffset=loff, tol=1e-10, relative=True, maxit=3000)
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    torch.cuda.synchronize()
    assert io["status"] == 0 and ig["status"] == 0
    assert abs(ig["res0"] - io["res0"]) <= 1e-12 * io["res0"]
    # Jacobi-PCG runs 100-450 iterations here; rounding differences (FMA contraction, reduction order)
    # may move the stopping iteration by one per hundred
    assert abs(ig["iterations"] - io["iterations"]) <= max(1, io["iterations"] // 100)
    assert rel(x.cpu().numpy(), xo) < 1e-7


def test_block_of_identical_fields_equals_scalar_solves(product_lib, torch_cuda):
    """Three copies of one right-hand side through the 3-field solver give three copies of the scalar
    Helmholtz solution (same operator per field; the block norm is the sum over the fields)."""
    torch = torch_cuda
    N, n = 5, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    s1 = G.Elliptic(N, VX, EToV, EToB, BASE.replace("pcg+block", "pcg") + ";lambda1=10.0;residualTol=1e-12")
    s3 = G.Elliptic(N, VX, EToV, EToB, BASE + ";lambda1=10.0;residualTol=1e-12")
    b = W.box_rhs(N, n, n, n, 8, s1.get("ggeo"))
    r1, x1 = torch.from_numpy(b.copy()).cuda(), torch.zeros(b.size, dtype=torch.float64, device="cuda")
    r3 = torch.from_numpy(np.concatenate([b, b, b])).cuda()
    x3 = torch.zeros_like(r3)
    i1, i3 = s1.solve(r1, x1), s3.solve(r3, x3)
    torch.cuda.synchronize()
    assert i1["status"] == 0 and i3["status"] == 0
    assert abs(i3["res0"] - np.sqrt(3) * i1["res0"]) <= 1e-12 * i3["res0"]
    xs = x3.cpu().numpy().reshape(3, -1)
    for f in range(3):
        assert rel(xs[f], x1.cpu().numpy()) < 1e-8


def test_block_rejects_multigrid_and_bad_field_counts(product_lib, torch_cuda):
    VX, EToV, EToB = W.kershaw_box(2, eps=0.3)
    with pytest.raises(G.NrsgError):
        G.Elliptic(3, VX, EToV, EToB, "solver=pcg+block;preconditioner=multigrid")
    with pytest.raises(G.NrsgError):
        G.Elliptic(3, VX, EToV, EToB, "solver=pcg;nFields=2;stressFormulation=true;preconditioner=jacobi")
    with pytest.raises(G.NrsgError):
        G.Elliptic(3, VX, EToV, EToB, "solver=pcg;nFields=4;preconditioner=jacobi")


@pytest.mark.parametrize("stress", [False, True])
def test_block_solve_with_per_field_boundary_types(product_lib, oracle_mod, torch_cuda, stress):
    """Boundary types per field (the reference's EToB with Nfields sections): the x-planes are symmetry-like,
    Dirichlet for the first component and Neumann for the other two; parity with the oracle, and the first
    component alone vanishes there."""
    torch = torch_cuda
    N, n = 5, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    E3 = np.stack([EToB.copy() for _ in range(3)])
    for f in (1, 2):
        for face in (2, 4):  # nekRS faces r+ and r-
            E3[f][:, face] = np.where(EToB[:, face] > 0, 4, 0)
    opts = BASE + ";lambda1=10.0;residualTol=1e-10+relative" + (";stressFormulation=true" if stress else "")
    orc = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    el.set_field_bcs(E3)
    rhs = np.concatenate([W.box_rhs(N, n, n, n, s, orc.get("ggeo")) for s in (11, 12, 13)])
    xo, io = orc.block_solve(rhs, nf=3, stress=stress, poisson=False, l0=1.0, l1=10.0, tol=1e-10, relative=True,
                             maxit=3000, EToB_fields=E3)
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    torch.cuda.synchronize()
    assert io["status"] == 0 and ig["status"] == 0
    assert abs(ig["res0"] - io["res0"]) <= 1e-12 * io["res0"]
    assert abs(ig["iterations"] - io["iterations"]) <= max(1, io["iterations"] // 100)
    xg = x.cpu().numpy()
    assert rel(xg, xo) < 1e-7
    xs = orc.get("x")
    on_x = np.isclose(xs, 0.0) | np.isclose(xs, 1.0)
    X = xg.reshape(3, -1)
    assert np.abs(X[0][on_x]).max() == 0.0 and np.abs(X[1][on_x]).max() > 0.0


def _rotation():
    a, b, c = 0.4, -0.7, 1.1
    Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
    Rz = np.array([[np.cos(c), -np.sin(c), 0], [np.sin(c), np.cos(c), 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def _zero_normal_x_planes(EToB):
    E3 = np.stack([EToB.copy() for _ in range(3)])
    for face in (2, 4):
        E3[:, :, face] = np.where(EToB[:, face] > 0, 2, 0)
    return E3


def _aligned_symmetry(EToB):
    E3 = np.stack([EToB.copy() for _ in range(3)])
    for f in (1, 2):
        for face in (2, 4):
            E3[f][:, face] = np.where(EToB[:, face] > 0, 4, 0)
    return E3


@pytest.mark.parametrize("N", [3, 5])
def test_zero_normal_block_solve(product_lib, oracle_mod, torch_cuda, N):
    """Zero-normal (symmetry) x-planes on a rotated Kershaw box (face type 2, ellipticApplyMask's
    applyZeroNormalMask): parity with the oracle's restatement, and the solution is R times the GPU solution of
    the unrotated problem with aligned symmetry planes (x-component Dirichlet, y and z Neumann)."""
    torch = torch_cuda
    n = 3
    R = _rotation()
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = BASE + ";lambda1=10.0;residualTol=1e-12+relative;maxIterations=5000"
    ali = G.Elliptic(N, VX, EToV, EToB, opts)
    rot = G.Elliptic(N, VX @ R.T, EToV, EToB, opts)
    orc = O.Elliptic(N, VX @ R.T, EToV, EToB, "preconditioner=jacobi")
    ali.set_field_bcs(_aligned_symmetry(EToB))
    rot.set_field_bcs(_zero_normal_x_planes(EToB))
    nl = orc.get("invDegree").size
    rhs = np.concatenate([W.box_rhs(N, n, n, n, s, orc.get("ggeo")) for s in (21, 22, 23)])
    rhs_rot = (R @ rhs.reshape(3, nl)).reshape(-1)
    out = {}
    for name, el, b in (("aligned", ali, rhs), ("rotated", rot, rhs_rot)):
        r = torch.from_numpy(b.copy()).cuda()
        x = torch.zeros_like(r)
        info = el.solve(r, x)
        torch.cuda.synchronize()
        assert info["status"] == 0
        out[name] = (info, x.cpu().numpy())
    xo, io = orc.block_solve(rhs_rot, nf=3, stress=False, poisson=False, l0=1.0, l1=10.0, tol=1e-12, relative=True,
                             maxit=5000, EToB_fields=_zero_normal_x_planes(EToB))
    ig, xg = out["rotated"]
    assert io["status"] == 0
    assert abs(ig["res0"] - io["res0"]) <= 1e-12 * io["res0"]
    assert abs(ig["iterations"] - io["iterations"]) <= max(1, io["iterations"] // 100)
    assert rel(xg, xo) < 1e-9
    want = (R @ out["aligned"][1].reshape(3, nl)).reshape(-1)
    err = rel(xg, want)
    print(f"N={N}: rotated zero-normal solve vs rotated aligned solve {err:.2e}; iterations GPU {ig['iterations']}, "
          f"oracle {io['iterations']}, aligned {out['aligned'][0]['iterations']}")
    assert err < 1e-9


def test_zero_normal_rejections(product_lib, torch_cuda):
    VX, EToV, EToB = W.kershaw_box(2, eps=0.3)
    el2 = G.Elliptic(3, VX, EToV, EToB, BASE.replace("pcg+block", "pcg") + ";nFields=2")
    with pytest.raises(G.NrsgError):
        el2.set_field_bcs(_zero_normal_x_planes(EToB)[:2])
    el3 = G.Elliptic(3, VX, EToV, EToB, BASE)
    E3 = _zero_normal_x_planes(EToB)
    E3[:, :, 0] = np.where(EToB[:, 0] > 0, 3, 0)  # zero-tangential
    with pytest.raises(G.NrsgError):
        el3.set_field_bcs(E3)


def test_zero_normal_stress_block_solve(product_lib, oracle_mod, torch_cuda):
    """Zero-normal x-planes with the stress (symmetric gradient) block operator: parity with the oracle's
    restatement (the rotation identity of the test above does not apply: the stress operator's Jacobi diagonal
    differs per component, and as in the reference the preconditioned vector is not projected)."""
    torch = torch_cuda
    N, n = 3, 3
    R = _rotation()
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = BASE + ";lambda1=10.0;residualTol=1e-10+relative;maxIterations=5000;stressFormulation=true"
    el = G.Elliptic(N, VX @ R.T, EToV, EToB, opts)
    orc = O.Elliptic(N, VX @ R.T, EToV, EToB, "preconditioner=jacobi")
    E3 = _zero_normal_x_planes(EToB)
    el.set_field_bcs(E3)
    rhs = np.concatenate([W.box_rhs(N, n, n, n, s, orc.get("ggeo")) for s in (31, 32, 33)])
    r = torch.from_numpy(rhs.copy()).cuda()
    x = torch.zeros_like(r)
    ig = el.solve(r, x)
    torch.cuda.synchronize()
    xo, io = orc.block_solve(rhs, nf=3, stress=True, poisson=False, l0=1.0, l1=10.0, tol=1e-10, relative=True,
                             maxit=5000, EToB_fields=E3)
    assert ig["status"] == 0 and io["status"] == 0
    assert abs(ig["res0"] - io["res0"]) <= 1e-12 * io["res0"]
    assert abs(ig["iterations"] - io["iterations"]) <= max(1, io["iterations"] // 100)
    assert rel(x.cpu().numpy(), xo) < 1e-7
