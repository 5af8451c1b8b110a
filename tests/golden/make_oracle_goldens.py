"""Writes oracle_goldens.json: SHA-256 digests of the float32 oracle's output after 6 steps of the
seeded step cases (every lattice x streaming method x storage x collision operator x LES, cases
'mixed' and 'ldc', on grids with non-power-of-two tiles), with digests of their inputs.  The CUDA
kernels are compared with the oracle on the same recipe (tests/test_gpu_step.py), so these digests
pin both.  Regenerate after a deliberate change to the oracle or to the case recipe:

    python tests/golden/make_oracle_goldens.py
"""
from __future__ import annotations

import itertools
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from mojo_lbm_gb300 import LBM_method  # noqa: E402
from tests.lbm_cases import digest, step_case  # noqa: E402

OUT = Path(__file__).with_name("oracle_goldens.json")
STEPS = 6
SHAPES = {"D2Q9": ((30, 20, 1), (10, 5, 1)), "D3Q19": ((18, 12, 10), (6, 4, 5)), "D3Q27": ((12, 12, 10), (4, 6, 5))}
CASES = list(itertools.product(["D2Q9", "D3Q19", "D3Q27"], ["db", "eso"], ["fp32", "f16c"],
                               ["SRT", "TRT", "KBC", "RLBM"], [False, True], ["mixed", "ldc"]))


def case_id(c) -> str:
    return "-".join(map(str, c))


def run_case(c):
    """(input digest, output digest) of one case: f after STEPS oracle steps and the bc array
    (captured rho / u land there)."""
    lat, meth, store, coll, les, kind = c
    grid, cfg, flags, bc, f0, tau = step_case(lat, meth, store, coll, les, kind, *SHAPES[lat])
    d_in = digest(f0, flags, bc, np.float32(tau))
    f, f2, bco = f0.copy(), f0.copy(), bc.copy()
    for k in range(STEPS):
        if cfg.lbm_method == LBM_method.DOUBLE_BUFFER:
            oracle.step(cfg, grid, 32, f2, f, bco, flags, tau)
            f, f2 = f2, f
        else:
            oracle.step(cfg, grid, 32, f, f, bco, flags, tau, k % 2 == 0)
    return d_in, digest(f, bco)


def main():
    out = {"steps": STEPS, "shapes": {k: [list(s), list(t)] for k, (s, t) in SHAPES.items()}, "cases": {}}
    for c in CASES:
        d_in, d_out = run_case(c)
        out["cases"][case_id(c)] = {"inputs": d_in, "outputs": d_out}
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(CASES)} cases to {OUT}")


if __name__ == "__main__":
    main()
