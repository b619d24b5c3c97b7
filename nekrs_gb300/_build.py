"""In-tree build of the nekrs_gb300 CUDA library for sm_103a.

Each translation unit under nekrs_gb300/csrc is compiled by its own nvcc
process (in parallel), then linked into nekrs_gb300/_lib/libnekrs_gb300.so.
Rebuilds only what changed.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
INC = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libnekrs_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction (-ffp-contract=off) so
# that host-side FP64 setup (basis, Givens rotations, projection scalars) rounds
# the same way on every host architecture.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I", INC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(SRC, "*.cu")) + glob.glob(os.path.join(SRC, "*.cpp")))
    hdrs = sorted(glob.glob(os.path.join(SRC, "*.hpp")) + glob.glob(os.path.join(INC, "*.h")))
    newest_hdr = max(os.path.getmtime(h) for h in hdrs)
    nvcc = _nvcc()
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if not force and os.path.exists(o) and os.path.getmtime(o) > max(os.path.getmtime(s), newest_hdr):
            continue
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
        if s.endswith(".cpp"):
            cmd = [nvcc] + NVCC_FLAGS + ["-x", "cu"] + ARCH + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd))
        procs.append((s, subprocess.Popen(cmd)))
    bad = [s for s, p in procs if p.wait() != 0]
    if bad:
        raise RuntimeError("nvcc failed for: " + ", ".join(bad))
    if force or procs or not os.path.exists(LIB):
        subprocess.check_call([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs + ["-lcudart"])
        _check_unresolved()
    return LIB


def _check_unresolved():
    """Fail the build if the library references a library-internal symbol it does not define."""
    try:
        out = subprocess.run(["nm", "-D", "--undefined-only", LIB], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        return
    missing = [ln.split()[-1] for ln in out.splitlines() if "nrsg" in ln]
    if missing:
        os.remove(LIB)
        raise RuntimeError("unresolved library symbols: " + ", ".join(missing))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
