"""TEST INFRASTRUCTURE: how fast the C restatement runs against OpenVort's
own build, at equal threads, on the 65,536-node velocity workload.

The CPU baseline timed beside the GPU must run where OpenVort's sources are
absent, so it runs the restatement (oracle/ov_oracle.c, built -O3:
_build/libovoracle_fast.so).  This script times one full update_tangle
(update_tangents_normals + update_velocities) of the same tangle in both
builds - the reference compiled from its own sources by `make ref`
(oracle/_ref/libovref.so, -O2 as the parity build) and, for comparison, the
restatement at the same -O2 - and writes the ratios to
oracle/port_vs_reference.json, which bench.py reports beside its CPU
baseline.  Run it where the OpenVort checkout exists:

    python oracle/port_vs_reference.py [threads]
"""
from __future__ import annotations

import json
import os
import platform
import statistics
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from openvort_gb300 import workloads as W  # noqa: E402
from oracle.pyoracle import Checker, build  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "port_vs_reference.json")


def time_update_tangle(checker, ht, p, reps):
    checker.set_params(p)
    ts = []
    for _ in range(reps):
        t = checker.tangle(ht)
        t0 = time.perf_counter()
        checker.update_tangle(t, 0.0)
        ts.append(time.perf_counter() - t0)
        t.free()
    return statistics.median(ts)


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    build(ref=True)
    ht = W.random_walk_tangle(256, 256, D=0.1, delta=1e-3, sigma=0.3, seed=1)
    p = W.config_params("rw", bh_resolution=0.4)
    p.num_threads = threads
    ref = time_update_tangle(Checker("reference"), ht, p, 3)
    port_fast = time_update_tangle(Checker("port", fast=True), ht, p, 3)
    port_parity = time_update_tangle(Checker("port", fast=False), ht, p, 3)
    n = ht.n
    out = {
        "workload": "one update_tangle of the 65,536-node random-walk tangle (256 loops x 256, D=0.1 cm, "
                    "theta 0.4, periodic_26)",
        "threads": threads, "machine": f"{platform.machine()}, {os.cpu_count()} cores",
        "reference_node_evals_per_s": n / ref,
        "port_fast_node_evals_per_s": n / port_fast,
        "port_parity_node_evals_per_s": n / port_parity,
        "port_over_reference": ref / port_fast,
        "port_parity_over_reference": ref / port_parity,
        "builds": "reference: OpenVort's sources, gcc -O2 -ffp-contract=off -fopenmp (octree.c with zm.h); "
                  "port: oracle/ov_oracle.c, gcc -O3 -fopenmp (fast) and the reference's -O2 flags (parity)",
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
