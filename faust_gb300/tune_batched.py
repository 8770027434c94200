"""Offline sweep for the batched palm4msa2 launch (run on the target GPU).

For batches whose largest dimension falls in each bucket (64, 128, 256, 512),
the batched launch is timed with 1, 2 and 3 resident CTAs per SM: with 1 a
CTA has the SM's whole shared memory for its staging area, with 2 the
128-register kernel runs, with 3 the kernel variant cut to 80 registers
runs.  The fastest choice per bucket goes to a JSON table that
fact.palm4msa_batched reads when ctas_per_sm is 0:

    python -m faust_gb300.tune_batched --out faust_gb300/tuning/batched_palm.json

Batches follow the batched workload's shape: n = round16(exp(U[ln lo,
ln maxdim])), two seeded batches per bucket, targets P1 P2 P3 + 1e-3 noise, 4 splincol factors with k = 4,
FP32 with FP64 step-size norms; `--its` iterations (the ranking of the
choices does not depend on the iteration count, so the sweep runs fewer than
the workload's 100).
"""
import argparse
import json
import os
import time

import numpy as np


def _batch(rng, count, lo, hi):
    from . import synth
    ns = (np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)) / 16) * 16).astype(int)
    ns = np.clip(ns, lo, hi)
    mats = []
    for n in ns:
        P = [synth.random_csr(int(n), int(n), 4, rng, np.float64) for _ in range(3)]
        A = (P[0] @ (P[1] @ P[2].toarray())) + 1e-3 * rng.standard_normal((n, n))
        mats.append(np.asarray(A, np.float32))
    return ns, mats


def sweep(count=512, its=30, reps=3, buckets=(64, 128, 256, 512), choices=(1, 2, 3), log=print):
    import torch
    from . import fact
    table = []
    for maxdim in buckets:
        # two batches per bucket (the makespan depends on the batch's mix of
        # sizes); a choice's time is the sum of its medians over both
        batches = []
        for seed in (maxdim, maxdim + 1):
            ns, mats = _batch(np.random.default_rng(seed), count, min(64, maxdim), maxdim)
            cons_by_n = {}
            probs = []
            for A, n in zip(mats, ns):
                if n not in cons_by_n:
                    cons_by_n[n] = [fact.ConstraintInt("splincol", int(n), int(n), 4) for _ in range(4)]
                probs.append((torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t(), cons_by_n[n]))
            batches.append(probs)
        params = fact.ParamsPalm4MSA(batches[0][0][1], its, norm2_fp64=True)
        times = {}
        for c in choices:
            total = 0.0
            for probs in batches:
                for r in fact.palm4msa_batched(probs[:64], params, ctas_per_sm=c):
                    r.faust.close()
                ts = []
                for _ in range(reps):
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    res = fact.palm4msa_batched(probs, params, ctas_per_sm=c)
                    ts.append(time.perf_counter() - t0)
                    for r in res:
                        r.faust.close()
                total += float(np.median(ts))
            times[c] = total
            log("maxdim %d, %d CTAs per SM: %.4f s (two batches)" % (maxdim, c, times[c]))
        best = min(times, key=times.get)
        table.append({"maxdim": int(maxdim), "ctas_per_sm": int(best),
                      "seconds": {str(k): round(v, 5) for k, v in times.items()}})
    return table


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning",
                                                  "batched_palm.json"))
    ap.add_argument("--count", type=int, default=512)
    ap.add_argument("--its", type=int, default=30)
    a = ap.parse_args()
    import torch
    table = sweep(a.count, a.its)
    out = {"f32": table,
           "device": torch.cuda.get_device_name(0),
           "how": "sum over two seeded batches of the median of 3 batched launches of %d instances per bucket, "
                  "%d iterations, splincol k=4, FP32 with FP64 norms; written by faust_gb300/tune_batched.py"
                  % (a.count, a.its)}
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
