"""Build recipe for the oracle (test infrastructure only).

Compiles the C++ restatement in oracle/*.cpp into oracle/_build/liboracle.so
with the host compiler (portable flags, no -march), and, when the reference
tree is present, the reference's serial kernels into oracle/_ref.
"""
import glob
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


def _fp_flags():
    """No floating-point contraction: the oracle rounds the same way on every
    host, with fused multiply-adds only where the source calls std::fma.  On
    x86-64 hosts whose CPU has FMA, -mfma lets those calls compile to the
    instruction instead of a library call (same result, correctly rounded)."""
    flags = ["-ffp-contract=off"]
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            with open("/proc/cpuinfo") as f:
                if " fma " in f.read():
                    flags.append("-mfma")
        except OSError:
            pass
    return flags


FP_FLAGS = _fp_flags()


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    lib = os.path.join(BUILD, "liboracle.so")
    srcs = sorted(glob.glob(os.path.join(HERE, "*.cpp")))
    hdrs = sorted(glob.glob(os.path.join(HERE, "*.hpp")))
    if not force and os.path.exists(lib):
        t = os.path.getmtime(lib)
        if all(os.path.getmtime(s) < t for s in srcs + hdrs):
            return lib
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-4] + ".o")
        objs.append(o)
        procs.append(subprocess.Popen(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC"] + FP_FLAGS + ["-c", s, "-o", o]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed")
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", lib] + objs)
    return lib


def build_all(reference_root=None):
    from . import build_ref  # noqa: E402

    lib = build_oracle()
    ref = None
    reference_root = reference_root or build_ref.reference_root()
    if os.path.isdir(reference_root):
        ref = build_ref.build(reference_root)
    return lib, ref


if __name__ == "__main__":
    print(build_all())
