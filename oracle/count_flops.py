"""Algorithmic operation counts of the reference algorithm per cell-update.

Runs the oracle on its counting scalar (every add/sub, mul, div, sqrt and
comparison of the Rust core is tallied once, as the reference evaluates it) for
each residual variant on a 64 x 64 interior, and writes the per-cell figures to
profiles/flops_per_cell.json.  One SSP-RK3 cell-update = 3 residuals + the
stage combinations (12 flops per conserved component over 3 stages = 36) + the
CFL reduction (about 12 per cell).

    python oracle/count_flops.py
"""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path = [p for p in sys.path if os.path.abspath(p or ".") != os.path.dirname(os.path.abspath(__file__))]
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import oracle  # noqa: E402
from states import quadrant  # noqa: E402


def main():
    n = 64
    q = quadrant(np.random.default_rng(1), n, n)
    out = {"grid": f"{n}x{n} interior, four-quadrant state", "per_residual": {}}
    for cons, cname in ((False, "char"), (True, "cons")):
        for hlle, hname in ((True, "hlle"), (False, "blend")):
            t = oracle.count_l_local(q, 1.0 / n, 1.4, hlle, (0.2, 1.0), cons)
            per = {k: v / (n * n) for k, v in t.items()}
            per["flops"] = per["add"] + per["mul"] + per["div"] + per["sqrt"]
            out["per_residual"][f"{cname}_{hname}"] = per
            out[f"{cname}_{hname}_step"] = 3 * per["flops"] + 36 + 12
    path = os.path.join(ROOT, "profiles", "flops_per_cell.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
