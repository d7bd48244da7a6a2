"""Autotuner for the batched path's tile shapes.

Times every combination of the batch tunables on a sample of the batched
workload (seeded uneven lifted Swiss rolls, N ~ U[500, 20000], D in
{3, 16, 64, 128}, k in {8, 12, 16, 24, 32}), by replaying each candidate's CUDA
graph, and writes the table tapkee_gb300/tuning/gb300_batch.json that
tapkee_gb300.batch.default_tuning() reads:

  screen_qt[0]  query blocks of 128 rows per screen work item (padded dimension 64)
  lle_warps     warps (one problem row each) per block of the weight solve
  wide_lists    64 screened candidates per row for every k, or the smallest list

Usage:  python -m tapkee_gb300.autotune [--count 64] [--reps 5] [--out PATH]
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import time

from . import datasets
from .batch import TUNING_PATH, Batch

SPACE = {"screen_qt0": [1, 2], "lle_warps": [4, 8], "wide_lists": [0, 1]}


def candidates():
    for qt, lw, wl in itertools.product(SPACE["screen_qt0"], SPACE["lle_warps"], SPACE["wide_lists"]):
        yield {"screen_qt": [qt, 1], "lle_warps": lw, "wide_lists": wl}


def tune(count=64, reps=5, seed=1234, context=None):
    import torch
    specs = datasets.batch_problems(count, seed=seed)
    Xs = [torch.from_numpy(datasets.batch_problem_data(n, d, s)).cuda() for n, d, k, s in specs]
    ks = [k for _, _, k, _ in specs]
    results = []
    for cand in candidates():
        b = Batch(Xs, ks, tuning=cand, context=context)
        b.run()
        ms = [b.run() for _ in range(reps)]
        b.close()
        results.append({"tuning": cand, "ms_median": statistics.median(ms), "ms_all": ms})
    best = min(results, key=lambda r: r["ms_median"])
    return {
        "device": torch.cuda.get_device_name(0),
        "workload": f"{count} problems, datasets.batch_problems(count, seed={seed}): N~U[500,20000], "
                    "D in {3,16,64,128}, k in {8,12,16,24,32}, float32",
        "points": int(sum(n for n, _, _, _ in specs)),
        "reps": reps,
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
        "results": results,
        "best": best["tuning"],
        "best_ms": best["ms_median"],
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out", default=TUNING_PATH)
    args = ap.parse_args()
    table = tune(args.count, args.reps)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps({"best": table["best"], "best_ms": table["best_ms"]}))


if __name__ == "__main__":
    main()
