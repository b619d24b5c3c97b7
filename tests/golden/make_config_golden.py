"""Generate tests/golden/config_parity.json: the oracle's solves of the two
configurations the headline metric is defined against, for the GPU parity
tests in tests/test_gpu_configs.py.

  c0  Kershaw box E=8^3, N=7, eps=0.3, Poisson, homogeneous Dirichlet, seeded
      mass-weighted U[-1,1] right-hand side, FP64 Jacobi-PCG to 1e-8 relative;
  c1  Kershaw box E=32^3, N=7, eps=0.3, same right-hand side recipe, plain FP64
      p-multigrid flexible PCG: levels 7/3/1, Chebyshev(2) over the overlapping
      Schwarz (fused FDM) smoother, coarse order-1 level by Jacobi-PCG to 1e-4,
      stored FP64 geometric factors, to 1e-8 relative.

For each: iteration count, res0 and final residual norm, the residual history,
and the solution's norm, SHA-256 of its bytes and its projections onto four
seeded U[-1,1] vectors.  Runs the CPU oracle only (a few minutes for c1):

    python tests/golden/make_config_golden.py
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nekrs_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "config_parity.json")

PMG = ("preconditioner=multigrid;smootherType=cheby+asm;"
       "pMGSchedule=p=7+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=7+degree=2;coarseSolver=jpcg;coarseTol=1e-4")
CONFIGS = {
    "c0": {"nel": 8, "N": 7, "eps": 0.3, "seed": 1234,
           "options": "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;maxIterations=20000"},
    "c1": {"nel": 32, "N": 7, "eps": 0.3, "seed": 1234,
           "options": "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG +
                      ";mgPrecision=fp64;axPrecision=fp64"},
}


def projections(x, k=4):
    """x . v_j for four seeded U[-1,1] vectors v_j."""
    return [float(np.dot(x, np.random.default_rng(7 + j).uniform(-1, 1, x.size))) for j in range(k)]


def solve(cfg):
    nel, N = cfg["nel"], cfg["N"]
    VX, EToV, EToB = W.kershaw_box(nel, eps=cfg["eps"])
    orc = O.Elliptic(N, VX, EToV, EToB, cfg["options"])
    rhs = W.box_rhs(N, nel, nel, nel, cfg["seed"], orc.get("ggeo"))
    x, info = orc.solve(rhs)
    return x, info


def main():
    out = {}
    for name, cfg in CONFIGS.items():
        t = time.perf_counter()
        x, info = solve(cfg)
        dt = time.perf_counter() - t
        out[name] = dict(cfg, iterations=int(info["iterations"]), status=int(info["status"]),
                         res0=float(info["res0"]), res=float(info["res"]),
                         history=[float(v) for v in info["history"]],
                         x_norm=float(np.linalg.norm(x)), x_sha256=hashlib.sha256(x.tobytes()).hexdigest(),
                         x_proj=projections(x), oracle_seconds=round(dt, 1))
        print(name, out[name]["iterations"], f"{dt:.1f} s", flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
