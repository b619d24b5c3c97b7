"""Host-side checks that need no GPU: the C ABI library loads and exports every
declared symbol; the library's setup maps are bit-identical to the oracle's;
the synthetic workload generator matches the oracle's."""
import ctypes
import os
import re

import numpy as np
import pytest

import nekrs_gb300 as G
from nekrs_gb300 import workloads as W
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\**\s*\**(nrsg_[a-z0-9_]+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_declared_symbols(product_lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(product_lib, n), n


def test_library_is_sm103a_build():
    from nekrs_gb300 import _build

    assert "arch=compute_103a,code=sm_103a" in _build.ARCH


@pytest.mark.parametrize("N,n,eps", [(1, 3, 0.3), (2, 2, 0.3), (3, 3, 1.0), (5, 3, 0.3), (7, 3, 0.3), (9, 2, 0.5)])
def test_setup_maps_bitexact_vs_oracle(product_lib, oracle_mod, N, n, eps):
    VX, EToV, EToB = W.kershaw_box(n, eps=eps)
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    m = G.host_setup_maps(N, EToV, EToB)
    for k in ("ids", "maskedIds", "gsOff", "gsIds", "maskIds"):
        assert np.array_equal(m[k], el.get(k)), k
    assert np.array_equal(m["invDegree"], el.get("invDegree"))


@pytest.mark.parametrize("z_bc", [1, 4])
def test_setup_maps_axis_fan(product_lib, oracle_mod, z_bc):
    """Twelve sectors around an axis, two layers: axis edges shared by 12 elements and the interior axis
    vertex by 24 (the box meshes stop at 4 and 8); numbering, gather groups and mask bit-exact."""
    VX, EToV, EToB = W.axis_fan(12, 2, z_bc=z_bc)
    N = 4
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    m = G.host_setup_maps(N, EToV, EToB)
    for k in ("ids", "maskedIds", "gsOff", "gsIds", "maskIds"):
        assert np.array_equal(m[k], el.get(k)), k
    sizes = np.diff(m["gsOff"])
    assert sizes.max() == 24 and (sizes == 12).sum() >= 6  # the z = 1 axis vertex; axis edge nodes


def test_setup_maps_mixed_boundaries(product_lib, oracle_mod):
    # Neumann faces and an interior-only mask pattern
    VX, EToV, EToB = W.kershaw_box(3, 2, 2, eps=0.3, all_dirichlet=False)
    EToB = EToB.copy()
    EToB[0, 4] = 1  # one Dirichlet face
    N = 4
    el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    m = G.host_setup_maps(N, EToV, EToB)
    for k in ("ids", "maskedIds", "gsOff", "gsIds", "maskIds"):
        assert np.array_equal(m[k], el.get(k)), k
    # one face of Dirichlet nodes; its edge and corner nodes are also masked in the neighbours' copies
    assert len(np.unique(m["ids"][m["maskIds"]])) == (N + 1) ** 2
    assert len(m["maskIds"]) == (N + 1) ** 2 + 2 * (N + 1) + 1


def test_single_element(product_lib, oracle_mod):
    VX, EToV, EToB = W.kershaw_box(1, eps=0.3)
    for N in (1, 2, 7):
        m = G.host_setup_maps(N, EToV, EToB)
        el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
        assert np.array_equal(m["gsIds"], el.get("gsIds"))
        # every node but the interior is on the boundary of a single element box
        assert len(m["maskIds"]) == (N + 1) ** 3 - max(N - 1, 0) ** 3


@pytest.mark.parametrize("eps", [0.3, 1.0])
def test_workload_mesh_and_rhs_match_oracle(oracle_mod, eps):
    for (N, n) in [(3, 4), (7, 3)]:
        VX, EToV, EToB = W.kershaw_box(n, eps=eps)
        VX2, EToV2, EToB2 = O.box_mesh(n, n, n, eps)
        assert np.array_equal(VX, VX2) and np.array_equal(EToV, EToV2) and np.array_equal(EToB, EToB2)
        el = O.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
        g = el.get("ggeo")
        assert np.array_equal(W.box_rhs(N, n, n, n, 99, g), O.box_rhs(N, n, n, n, 99, g))


def test_rhs_is_continuous(oracle_mod):
    N, n = 5, 3
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    ids = G.host_setup_maps(N, EToV, EToB)["ids"]
    f = W.box_field(N, n, n, n, 5)
    assert f.min() >= -1 and f.max() <= 1
    nz = ids != 0
    order = np.argsort(ids[nz], kind="stable")
    s_ids, s_f = ids[nz][order], f[nz][order]
    same = s_ids[1:] == s_ids[:-1]
    assert np.array_equal(s_f[1:][same], s_f[:-1][same])


def test_kernel_launch_counter_available(product_lib):
    assert G.kernel_launches() >= 0
