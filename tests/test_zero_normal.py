"""Zero-normal (symmetry) boundaries of any orientation, face type 2, for the
three-field block solve: the oracle's restatement checked on the CPU.

On a Kershaw box rotated by R, with the x-planes zero-normal and the other
faces Dirichlet: (1) the averaged node normals of the x-planes are +-R e_x
and the frames are orthonormal; (2) the projection removes exactly the normal
component at zero-normal nodes and leaves Dirichlet-type nodes unchanged; (3)
the rotated problem's solution is R times the solution of the unrotated
problem with the x-planes aligned-symmetric (x-component Dirichlet, y and z
components Neumann) — a check that needs neither the reference nor the
product."""
import numpy as np
import pytest

from nekrs_gb300 import workloads as W
from oracle import oracle as O


def rotation():
    a, b, c = 0.4, -0.7, 1.1
    Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
    Rz = np.array([[np.cos(c), -np.sin(c), 0], [np.sin(c), np.cos(c), 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def symmetric_x_planes(EToB):
    """x-planes (nekRS faces r+ = 2, r- = 4) zero-normal for every field, other boundary faces Dirichlet."""
    E3 = np.stack([EToB.copy() for _ in range(3)])
    for face in (2, 4):
        E3[:, :, face] = np.where(EToB[:, face] > 0, 2, 0)
    return E3


def aligned_symmetry(EToB):
    """the same boundaries with the x-planes axis-aligned symmetric: x-component Dirichlet, y, z Neumann"""
    E3 = np.stack([EToB.copy() for _ in range(3)])
    for f in (1, 2):
        for face in (2, 4):
            E3[f][:, face] = np.where(EToB[:, face] > 0, 4, 0)
    return E3


def rotate_fields(R, U, nl):
    X = np.asarray(U).reshape(3, nl)
    return (R @ X).reshape(-1)


@pytest.mark.parametrize("N", [3, 5])
def test_zero_normal_frames_on_rotated_box(oracle_mod, N):
    n = 3
    R = rotation()
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    VXr = VX @ R.T
    orc = O.Elliptic(N, VXr, EToV, EToB, "preconditioner=jacobi")
    E3 = symmetric_x_planes(EToB)
    sgeo, mask = orc.zero_normal(E3[0])
    nq = N + 1
    ex = R @ np.array([1.0, 0.0, 0.0])
    for face, sign in ((2, 1.0), (4, -1.0)):
        els = np.nonzero(EToB[:, face] > 0)[0]
        fr = sgeo[els, face]  # [e][nq^2][9]
        nrm, t1, t2 = fr[..., 0:3], fr[..., 3:6], fr[..., 6:9]
        assert np.abs(nrm - sign * ex).max() < 1e-13
        for a, b in ((nrm, t1), (nrm, t2), (t1, t2)):
            assert np.abs((a * b).sum(-1)).max() < 1e-13
        for a in (t1, t2):
            assert np.abs(np.linalg.norm(a, axis=-1) - 1).max() < 1e-13
    # faces that are not zero-normal carry no frame
    assert np.abs(sgeo[:, [0, 1, 3, 5]]).max() == 0.0
    # mask: maskN = 0 exactly on x-plane nodes that touch no Dirichlet face
    x, y, z = (orc.get(k) for k in ("x", "y", "z"))
    xs_ref = (R.T @ np.stack([x, y, z])).T  # back to the unrotated box
    on_x = np.isclose(xs_ref[:, 0], 0) | np.isclose(xs_ref[:, 0], 1)
    on_other = (np.isclose(xs_ref[:, 1], 0) | np.isclose(xs_ref[:, 1], 1) | np.isclose(xs_ref[:, 2], 0)
                | np.isclose(xs_ref[:, 2], 1))
    nl = x.size
    mN = mask[:nl]
    assert np.all(mN[on_x & ~on_other] == 0.0)
    assert np.all(mN[~(on_x & ~on_other)] == 1.0)
    assert np.all(mask[nl:] == 1.0)


def test_zero_normal_projection(oracle_mod):
    N, n = 4, 3
    R = rotation()
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    orc = O.Elliptic(N, VX @ R.T, EToV, EToB, "preconditioner=jacobi")
    E3 = symmetric_x_planes(EToB)
    x, y, z = (orc.get(k) for k in ("x", "y", "z"))
    nl = x.size
    U = np.random.default_rng(4).standard_normal(3 * nl)
    V = orc.apply_zero_normal(E3[0], U)
    xs_ref = (R.T @ np.stack([x, y, z])).T
    on_x = np.isclose(xs_ref[:, 0], 0) | np.isclose(xs_ref[:, 0], 1)
    on_other = (np.isclose(xs_ref[:, 1], 0) | np.isclose(xs_ref[:, 1], 1) | np.isclose(xs_ref[:, 2], 0)
                | np.isclose(xs_ref[:, 2], 1))
    zn = on_x & ~on_other
    ex = R @ np.array([1.0, 0.0, 0.0])
    Uf, Vf = U.reshape(3, nl), V.reshape(3, nl)
    # normal component removed, tangential part kept
    # (the averaged normals equal R e_x to ~1e-13, the field values are O(1))
    assert np.abs(ex @ Vf[:, zn]).max() < 1e-12
    tang = Uf[:, zn] - np.outer(ex, ex @ Uf[:, zn])
    assert np.abs(Vf[:, zn] - tang).max() < 1e-12
    # nodes on no zero-normal face untouched; Dirichlet-type x-plane nodes kept up to rounding
    assert np.array_equal(Vf[:, ~on_x], Uf[:, ~on_x])
    assert np.abs(Vf[:, on_x & on_other] - Uf[:, on_x & on_other]).max() < 1e-12


def test_rotated_symmetry_solve_equals_rotated_aligned_solve(oracle_mod):
    N, n = 3, 3
    R = rotation()
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    ali = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    rot = O.Elliptic(N, VX @ R.T, EToV, EToB, "preconditioner=jacobi")
    nl = ali.get("invDegree").size
    rhs = np.concatenate([W.box_rhs(N, n, n, n, s, ali.get("ggeo")) for s in (21, 22, 23)])
    kw = dict(nf=3, stress=False, poisson=False, l0=1.0, l1=10.0, tol=1e-12, relative=True, maxit=5000)
    xa, ia = ali.block_solve(rhs, EToB_fields=aligned_symmetry(EToB), **kw)
    xr, ir = rot.block_solve(rotate_fields(R, rhs, nl), EToB_fields=symmetric_x_planes(EToB), **kw)
    assert ia["status"] == 0 and ir["status"] == 0
    want = rotate_fields(R, xa, nl)
    err = np.abs(xr - want).max() / np.abs(want).max()
    print(f"rotated symmetric solve vs rotated aligned solve: {err:.2e} ({ir['iterations']} / {ia['iterations']} it)")
    assert err < 1e-9
