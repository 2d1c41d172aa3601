"""Autotuner for the kernel variants of libvkhel on the running GPU.

    python -m vkhel_gb300.autotune            # writes vkhel_gb300/tuning/gb300.txt (+ _report.json)

For every CTA-resident degree 2^8 .. 2^14 it times each compiled variant
(words per thread, radix-16 groups in flight per thread) of the fused
polymul, the forward and the inverse transform on a batch that fills the GPU
several times over (one limb job per polynomial, a 60-bit prime, uniform
operands), and for ragged batches it times running the degree classes
sequentially against running them on concurrent streams.  The
fastest choice of each is written to the table libvkhel reads at start-up
(see vkhel_tune_* in include/vkhel/vkhel_ext.h).  Every variant computes the
same words (tests/test_gpu_variants.py checks them against the oracle), so
the table changes speed only.
"""
import json
import os
import sys
import time

import numpy as np

import vkhel_gb300 as vk
from vkhel_gb300 import workloads

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning", "gb300.txt")
REPORT = os.path.join(HERE, "tuning", "gb300_report.json")

POLYMUL, FORWARD, INVERSE, BATCH = 0, 1, 2, 3
VARIANTS = {8: [0, 1], 9: [0, 1], 10: [0, 1, 2], 11: [0, 1, 2], 12: [0, 1, 2], 13: [0, 1, 2], 14: [0, 1]}
DESCRIBE = {0: "default shape", 1: "two radix-16 groups in flight per thread",
            2: "other words-per-thread shape"}


def _time_batch(ctx, bt, reps):
    bt.launch()
    bt.launch()
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        bt.launch()
    ctx.sync()
    return (time.perf_counter() - t0) / reps


def _single_limb_jobs(ctx, log_n, count, seed):
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1)[0]
    t = vk.NttTables(n, q, workloads.root_for(n, q))
    rng = np.random.default_rng(seed)
    a = vk.Vector(ctx, workloads.uniform(rng, q, count * n))
    b = vk.Vector(ctx, workloads.uniform(rng, q, count * n))
    c = vk.Vector(ctx, count * n)
    return t, a, b, c


def tune_polymul(ctx, sms, reps=30):
    L = vk.lib()
    best, report = {}, {}
    for log_n, variants in VARIANTS.items():
        n = 1 << log_n
        count = 4 * sms * max(1, (1 << 14) // n)
        t, a, b, c = _single_limb_jobs(ctx, log_n, count, seed=log_n)
        times = {}
        for v in variants:
            L.vkhel_tune_set(POLYMUL, log_n, v)
            bt = vk.Batch(ctx)
            for j in range(count):
                bt.add_polymul([t], a.device_ptr + 8 * j * n, b.device_ptr + 8 * j * n, c.device_ptr + 8 * j * n)
            bt.commit(graph=False)  # the variant is read at every launch
            times[v] = _time_batch(ctx, bt, reps)
            bt.close()
        v_best = min(times, key=times.get)
        L.vkhel_tune_set(POLYMUL, log_n, v_best)
        best[log_n] = v_best
        report[str(log_n)] = {"jobs": count, "seconds_per_batch": {str(k): x for k, x in times.items()},
                              "chosen": v_best, "chosen_is": DESCRIBE[v_best]}
        for x in (a, b, c):
            x.close()
    return best, report


def tune_transforms(ctx, sms, family, reps=30):
    """Variants of the forward (family 1) or inverse (family 2) transform."""
    L = vk.lib()
    best, report = {}, {}
    for log_n, variants in VARIANTS.items():
        n = 1 << log_n
        count = 4 * sms * max(1, (1 << 14) // n)
        t, a, b, c = _single_limb_jobs(ctx, log_n, count, seed=100 + log_n)
        times = {}
        for v in variants:
            L.vkhel_tune_set(family, log_n, v)
            bt = vk.Batch(ctx)
            bt.add_transform([t] * count, a, c, inverse=family == INVERSE)
            bt.commit(graph=False)  # the variant is read at every launch
            times[v] = _time_batch(ctx, bt, reps)
            bt.close()
        v_best = min(times, key=times.get)
        L.vkhel_tune_set(family, log_n, v_best)
        best[log_n] = v_best
        report[str(log_n)] = {"jobs": count, "seconds_per_batch": {str(k): x for k, x in times.items()},
                              "chosen": v_best, "chosen_is": DESCRIBE[v_best]}
        for x in (a, b, c):
            x.close()
    return best, report


def tune_concurrency(ctx, reps=5, instances=256):
    L = vk.lib()
    inst = workloads.ragged_instances(instances, seed=33)
    rng = np.random.default_rng(33)
    prim, jobs = {}, []
    for log_n, limbs in inst:
        n = 1 << log_n
        if n not in prim:
            qs = workloads.ntt_primes(n, 16)
            prim[n] = [vk.NttTables(n, q, workloads.root_for(n, q)) for q in qs]
        tl = prim[n][:limbs]
        qs = [x.q for x in tl]
        a = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        bb = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        jobs.append((tl, vk.Vector(ctx, a), vk.Vector(ctx, bb), vk.Vector(ctx, limbs * n)))
    times = {}
    for flag in (0, 1):
        L.vkhel_tune_set(BATCH, 0, flag)
        bt = vk.Batch(ctx)
        for tl, a, bb, c in jobs:
            bt.add_polymul(tl, a, bb, c)
        bt.commit(graph=True)
        times[flag] = _time_batch(ctx, bt, reps)
        bt.close()
    best = min(times, key=times.get)
    L.vkhel_tune_set(BATCH, 0, best)
    return best, {"instances": instances, "seconds_per_batch": {"sequential": times[0], "concurrent": times[1]},
                  "chosen": "concurrent" if best else "sequential"}


def main(argv):
    out_table = argv[0] if argv else TABLE
    # start from the built-in defaults, not from a previous table
    os.environ["VKHEL_TUNE_TABLE"] = ""
    ctx = vk.Context()
    sms = ctx.sm_count
    best, report = tune_polymul(ctx, sms)
    fwd, fwd_report = tune_transforms(ctx, sms, FORWARD)
    inv, inv_report = tune_transforms(ctx, sms, INVERSE)
    conc, conc_report = tune_concurrency(ctx)
    ctx.close()
    os.makedirs(os.path.dirname(out_table), exist_ok=True)
    lines = ["# vkhel kernel variants for NVIDIA GB300 (sm_103a), written by `python -m vkhel_gb300.autotune`",
             "# family log_n variant   (family 0 = fused polymul, 1 = forward, 2 = inverse;",
             "#                         family 3 log_n 0 = concurrent degree classes)"]
    lines += [f"{POLYMUL} {log_n} {v}" for log_n, v in sorted(best.items())]
    lines += [f"{FORWARD} {log_n} {v}" for log_n, v in sorted(fwd.items())]
    lines += [f"{INVERSE} {log_n} {v}" for log_n, v in sorted(inv.items())]
    lines += [f"{BATCH} 0 {conc}"]
    with open(out_table, "w") as f:
        f.write("\n".join(lines) + "\n")
    rep = {"gpu_sms": sms, "polymul": report, "forward": fwd_report, "inverse": inv_report,
           "batch_classes": conc_report,
           "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    with open(os.path.splitext(out_table)[0] + "_report.json", "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps({"table": out_table, "polymul": best, "forward": fwd, "inverse": inv,
                      "concurrent_classes": conc}))


if __name__ == "__main__":
    main(sys.argv[1:])
