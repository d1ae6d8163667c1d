"""Regenerate tests/golden/config1_oracle.json: the oracle's run of the headless
Plummer workload (N=1000, seed 42, eps=0.01, dt=1e-3, 10^4 KDK steps with the
serial symmetric BruteForce, crates/sim-core/src/gravity.rs:47-80 and
integrator.rs:42-76).  The run takes about half a minute on one core, so the
GPU test compares against these numbers instead of re-running it.

The oracle has no FMA contraction and uses only correctly rounded f64
operations, so the numbers are the same on every host architecture.

Usage: python tests/golden/make_config1.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402

N, SEED, EPS, DT, STEPS, EVERY = 1000, 42, 0.01, 1e-3, 10000, 1000


def state_hash(p) -> str:
    h = hashlib.sha256()
    for f in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
        h.update(np.ascontiguousarray(getattr(p, f), dtype="<f8").tobytes())
    return h.hexdigest()


def main() -> None:
    q = O.plummer(N, SEED)
    g = O.gravity(O.GRAV_BF, EPS)
    q.clear_accelerations()
    O.bf_serial(q, EPS)
    rows = []
    d = O.diagnostics(q, EPS)
    rows.append({"step": 0, "total_energy": d["total_energy"], "momentum": d["momentum_mag"],
                 "angular_momentum": d["angular_momentum_mag"], "state_sha256": state_hash(q)})
    for k in range(STEPS // EVERY):
        O.kdk_steps(q, g, DT, EVERY)
        d = O.diagnostics(q, EPS)
        rows.append({"step": (k + 1) * EVERY, "total_energy": d["total_energy"], "momentum": d["momentum_mag"],
                     "angular_momentum": d["angular_momentum_mag"], "state_sha256": state_hash(q)})
    out = {"workload": f"Plummer N={N} seed {SEED}, eps={EPS}, dt={DT}, {STEPS} KDK steps, serial BruteForce",
           "rows": rows, "x_final_first4": [float(v) for v in q.x[:4]]}
    dst = os.path.join(HERE, "config1_oracle.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main()
