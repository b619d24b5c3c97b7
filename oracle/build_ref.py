"""Build recipe for oracle/_ref: the reference's own serial CPU kernels.

Test infrastructure only.  Each kernel instance is compiled straight from
its source file under the reference tree (kernels/elliptic/*.c), with the
JIT-time macros (FUNC, p_Nq, p_Np, p_G**ID, p_poisson, p_lambda, dfloat,
pfloat, dlong, ...) supplied by a generated wrapper, into one shared library
oracle/_ref/libnekref.so.  Nothing from the reference is copied into the
repository; the wrappers and the library live in the git-ignored
oracle/_ref/ folder.  When the reference tree is absent (the GPU host) this
script does nothing and the parity tests that need it are skipped.

Usage: python oracle/build_ref.py [reference_root]   (default: $NEKRS_REFERENCE_ROOT)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

AX_ORDERS = [1, 2, 3, 4, 5, 6, 7, 8, 9]
TRANSFER_PAIRS = [(2, 1), (3, 1), (5, 3), (7, 3), (7, 5), (9, 5), (5, 1), (4, 2), (6, 3), (9, 7)]
FDM_ORDERS = [1, 2, 3, 4, 5, 6, 7, 8, 9]
BLOCK_ORDERS = [1, 3, 5, 7]


def _common(dfloat, pfloat):
    return [
        "#define dlong int",
        "#define hlong long long",
        f"#define dfloat {dfloat}",
        f"#define pfloat {pfloat}",
        "#define p_blockSize 256",
    ]


def _undef():
    names = ["FUNC", "dlong", "hlong", "dfloat", "pfloat", "p_blockSize", "p_Nq", "p_Np", "p_Nggeo",
             "p_G00ID", "p_G01ID", "p_G02ID", "p_G11ID", "p_G12ID", "p_G22ID", "p_GWJID", "p_lambda",
             "p_poisson", "p_knl", "p_NqFine", "p_NqCoarse", "p_NpFine", "p_NpCoarse", "p_Nq_e",
             "p_Np_e", "p_restrict", "p_Nfields", "p_Nvgeo", "p_RXID", "p_RYID", "p_RZID", "p_SXID", "p_SYID",
             "p_SZID", "p_TXID", "p_TYID", "p_TZID", "p_JWID"]
    return [f"#undef {n}" for n in names]


def wrappers(ref):
    ke = os.path.join(ref, "kernels", "elliptic")
    units = []
    # axhelm, stored geometric factors (mesh3D.h:96-102 ids)
    for N in AX_ORDERS:
        for prec, ty in (("d", "double"), ("f", "float")):
            for kind in ("p", "h"):
                lines = _common(ty, "float") + [
                    f"#define FUNC(a) ref_ax_{prec}_{kind}_N{N}",
                    "#define p_knl 0",
                    f"#define p_Nq {N + 1}",
                    f"#define p_Np {(N + 1) ** 3}",
                    "#define p_Nggeo 7",
                    "#define p_G00ID 0", "#define p_G01ID 1", "#define p_G11ID 2", "#define p_G12ID 3",
                    "#define p_G02ID 4", "#define p_G22ID 5", "#define p_GWJID 6",
                    "#define p_lambda 0",
                ]
                if kind == "p":
                    lines.append("#define p_poisson 1")
                lines.append(f'#include "{os.path.join(ke, "ellipticPartialAxCoeffHex3D.c")}"')
                lines += _undef()
                units.append("\n".join(lines))
    # p-multigrid restriction / prolongation
    for (Nf, Nc) in TRANSFER_PAIRS:
        for prec, ty in (("d", "double"), ("f", "float")):
            for kern in ("ellipticPreconCoarsenHex3D", "ellipticPreconProlongateHex3D"):
                short = "coarsen" if "Coarsen" in kern else "prolong"
                lines = _common("double", ty) + [
                    f"#define FUNC(a) ref_{short}_{prec}_{Nf}_{Nc}",
                    f"#define p_NqFine {Nf + 1}", f"#define p_NqCoarse {Nc + 1}",
                    f"#define p_NpFine {(Nf + 1) ** 3}", f"#define p_NpCoarse {(Nc + 1) ** 3}",
                    f'#include "{os.path.join(ke, kern + ".c")}"',
                ] + _undef()
                units.append("\n".join(lines))
    # FDM smoother kernels on the (N+3)^3 extended element
    for N in FDM_ORDERS:
        for prec, ty in (("d", "double"), ("f", "float")):
            base = _common("double", ty) + [f"#define p_Nq {N + 1}", f"#define p_Nq_e {N + 3}",
                                            f"#define p_Np_e {(N + 3) ** 3}"]
            units.append("\n".join(base + [f"#define FUNC(a) ref_prefdm_{prec}_N{N}",
                                           f'#include "{os.path.join(ke, "preFDM.c")}"'] + _undef()))
            units.append("\n".join(base + [f"#define FUNC(a) ref_postfdm_{prec}_N{N}",
                                           f'#include "{os.path.join(ke, "postFDM.c")}"'] + _undef()))
            for r in (0, 1):
                units.append("\n".join(base + [f"#define p_restrict {r}",
                                               f"#define FUNC(a) ref_fdm{'r' if r else 'a'}_{prec}_N{N}",
                                               f'#include "{os.path.join(ke, "fusedFDM.c")}"'] + _undef()))
    # axhelm with coefficient fields (p_lambda 1), Helmholtz
    for N in BLOCK_ORDERS:
        units.append("\n".join(_common("double", "float") + [
            f"#define FUNC(a) ref_axcoef_N{N}", "#define p_knl 0",
            f"#define p_Nq {N + 1}", f"#define p_Np {(N + 1) ** 3}", "#define p_Nggeo 7",
            "#define p_G00ID 0", "#define p_G01ID 1", "#define p_G11ID 2", "#define p_G12ID 3",
            "#define p_G02ID 4", "#define p_G22ID 5", "#define p_GWJID 6", "#define p_lambda 1",
            f'#include "{os.path.join(ke, "ellipticPartialAxCoeffHex3D.c")}"'] + _undef()))
    # block (3-field) and stress (symmetric-gradient) axhelm, scalar (p_lambda 0) and field coefficients
    for N in BLOCK_ORDERS:
        for lam in (0, 1):
            units.append("\n".join(_common("double", "float") + [
                f"#define FUNC(a) ref_block_l{lam}_N{N}", "#define p_knl 0",
                f"#define p_Nq {N + 1}", f"#define p_Np {(N + 1) ** 3}", "#define p_Nggeo 7",
                "#define p_G00ID 0", "#define p_G01ID 1", "#define p_G11ID 2", "#define p_G12ID 3",
                "#define p_G02ID 4", "#define p_G22ID 5", "#define p_GWJID 6", f"#define p_lambda {lam}",
                f'#include "{os.path.join(ke, "ellipticBlockPartialAxCoeffHex3D.c")}"'] + _undef()))
            units.append("\n".join(_common("double", "float") + [
                f"#define FUNC(a) ref_stress_l{lam}_N{N}", "#define p_knl 0",
                f"#define p_Nq {N + 1}", f"#define p_Np {(N + 1) ** 3}", "#define p_Nvgeo 12",
                "#define p_RXID 0", "#define p_RYID 1", "#define p_RZID 2", "#define p_SXID 3", "#define p_SYID 4",
                "#define p_SZID 5", "#define p_TXID 6", "#define p_TYID 7", "#define p_TZID 8", "#define p_JWID 10",
                f"#define p_lambda {lam}",
                f'#include "{os.path.join(ke, "ellipticStressPartialAxCoeffHex3D.c")}"'] + _undef()))
    # fused PCG residual update
    units.append("\n".join(_common("double", "float") + [
        "#define p_Nfields 1", "#define FUNC(a) ref_update_pcg",
        f'#include "{os.path.join(ke, "ellipticBlockUpdatePCG.c")}"'] + _undef()))
    return units


def reference_root():
    """Root of the reference source tree: $NEKRS_REFERENCE_ROOT, else where this
    build environment mounts it."""
    return os.environ.get("NEKRS_REFERENCE_ROOT", "/root/reference")


def build(ref=None):
    ref = ref or reference_root()
    if not os.path.isdir(os.path.join(ref, "kernels", "elliptic")):
        print("build_ref: reference tree not found, skipping")
        return None
    gen = os.path.join(OUT, "gen")
    os.makedirs(gen, exist_ok=True)
    srcs = []
    for i, text in enumerate(wrappers(ref)):
        p = os.path.join(gen, f"unit{i:03d}.cpp")
        if not os.path.exists(p) or open(p).read() != text:
            with open(p, "w") as f:
                f.write(text)
        srcs.append(p)
    # a handful of translation units, compiled in parallel
    groups = [srcs[i::8] for i in range(8)]
    objs, procs = [], []
    for gi, grp in enumerate(groups):
        agg = os.path.join(gen, f"group{gi}.cpp")
        with open(agg, "w") as f:
            f.write("".join(f'#include "{s}"\n' for s in grp))
        obj = os.path.join(gen, f"group{gi}.o")
        objs.append(obj)
        # no floating-point contraction: the kernels round as written on every host
        procs.append(subprocess.Popen(["g++", "-O2", "-fPIC", "-ffp-contract=off", "-c", agg, "-o", obj]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("build_ref: compile failed")
    lib = os.path.join(OUT, "libnekref.so")
    subprocess.check_call(["g++", "-shared", "-o", lib] + objs)
    return lib


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
