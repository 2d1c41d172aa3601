"""Autotuner for the kernel variants of libvkhel on the running GPU.

    python -m vkhel_gb300.autotune            # writes vkhel_gb300/tuning/gb300.txt (+ _report.json)

For every CTA-resident degree 2^8 .. 2^14 and every job-count bucket (jobs
per SM of the launch: at most 1, at most 2, at most 4, more) it times each
compiled variant (words per thread, radix-16 groups in flight per thread) of
the fused polymul, the forward and the inverse transform on a batch of that
many single-limb jobs (a 60-bit prime, uniform operands).  The variants
differ in threads per CTA and so in CTAs per SM, and a degree class's job
count (instances times limbs) decides how its last wave fills, so the choice
is made per (degree, job count) -- that is, per (N, limbs) of the workload.
For ragged batches it times running the degree classes sequentially, on
concurrent streams, and as one persistent launch over all classes.  The fastest choice of each is written
to the table libvkhel reads at start-up (see vkhel_tune_* in
include/vkhel/vkhel_ext.h).  Every variant computes the same words
(tests/test_gpu_variants.py checks them against the oracle), so the table
changes speed only.
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
# a variant replaces the incumbent (variant 0 for the many-jobs bucket, the
# many-jobs choice for the other buckets) only when it is this much faster:
# smaller gaps are within run-to-run noise
MARGIN = 0.02
# jobs per SM timed for each bucket of the table (<= 1, <= 2, <= 4, more)
BUCKET_JOBS_PER_SM = (1.0, 1.5, 3.0, 8.0)
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


def _tune_family(ctx, sms, family, reps):
    """Best variant per (degree, bucket) of the fused polymul (family 0) or
    the forward (1) / inverse (2) transform."""
    L = vk.lib()
    best, report = {}, {}
    for log_n, variants in VARIANTS.items():
        n = 1 << log_n
        counts = [max(1, int(round(k * sms))) for k in BUCKET_JOBS_PER_SM]
        # many jobs: several waves of the smaller shapes too
        counts[-1] = max(counts[-1], 4 * sms * max(1, (1 << 14) // n))
        t, a, b, c = _single_limb_jobs(ctx, log_n, counts[-1], seed=100 * family + log_n)
        incumbent = 0
        for bucket in reversed(range(len(counts))):
            count = counts[bucket]
            times = {}
            for v in variants:
                L.vkhel_tune_set(family, log_n, v)
                bt = vk.Batch(ctx)
                if family == POLYMUL:
                    for j in range(count):
                        bt.add_polymul([t], a.device_ptr + 8 * j * n, b.device_ptr + 8 * j * n,
                                       c.device_ptr + 8 * j * n)
                else:
                    bt.add_transform([t] * count, a, c, inverse=family == INVERSE)
                bt.commit(graph=False)  # the variant is read at every launch
                times[v] = _time_batch(ctx, bt, reps)
                bt.close()
            v_best = choose(times, incumbent)
            if bucket == len(counts) - 1:
                incumbent = v_best
            best[(log_n, bucket)] = v_best
            report[f"{log_n}/{bucket}"] = {"jobs": count, "seconds_per_batch": {str(k): x for k, x in times.items()},
                                           "chosen": v_best, "chosen_is": DESCRIBE[v_best]}
        for x in (a, b, c):
            x.close()
    for (log_n, bucket), v in best.items():  # leave the many-jobs choice set for the later families
        if bucket == len(BUCKET_JOBS_PER_SM) - 1:
            L.vkhel_tune_set(family, log_n, v)
    return best, report


def choose(times, incumbent):
    """The fastest variant, unless the incumbent is within MARGIN of it."""
    v = min(times, key=times.get)
    if incumbent in times and times[incumbent] <= times[v] * (1 + MARGIN):
        return incumbent
    return v


def table_from_report(report):
    """Re-derive the per-bucket choices of a saved report with choose()."""
    out = {}
    for fam_name, fam in (("polymul", POLYMUL), ("forward", FORWARD), ("inverse", INVERSE)):
        rows = report[fam_name]
        for log_n in sorted({int(k.split("/")[0]) for k in rows}):
            buckets = sorted(int(k.split("/")[1]) for k in rows if int(k.split("/")[0]) == log_n)
            incumbent = 0
            for b in reversed(buckets):
                times = {int(k): x for k, x in rows[f"{log_n}/{b}"]["seconds_per_batch"].items()}
                v = choose(times, incumbent)
                if b == buckets[-1]:
                    incumbent = v
                out[(fam, log_n, b)] = v
    return out


def tune_polymul(ctx, sms, reps=20):
    return _tune_family(ctx, sms, POLYMUL, reps)


def tune_transforms(ctx, sms, family, reps=20):
    return _tune_family(ctx, sms, family, reps)


def tune_concurrency(ctx, reps=5, instances=256):
    """Ragged batches (n = 2^12 .. 2^16, 1 .. 16 limbs): the degree classes one
    after another, on concurrent streams, or all in one persistent launch."""
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
    for name, concurrent, single in (("sequential", 0, 0), ("concurrent", 1, 0), ("single_launch", 0, 1)):
        L.vkhel_tune_set(BATCH, 0, concurrent)
        L.vkhel_tune_set(BATCH, 2, single)
        bt = vk.Batch(ctx)
        for tl, a, bb, c in jobs:
            bt.add_polymul(tl, a, bb, c)
        bt.commit(graph=True)
        times[name] = _time_batch(ctx, bt, reps)
        bt.close()
    best = min(times, key=times.get)
    L.vkhel_tune_set(BATCH, 0, 1 if best == "concurrent" else 0)
    L.vkhel_tune_set(BATCH, 2, 1 if best == "single_launch" else 0)
    return best, {"instances": instances, "seconds_per_batch": times, "chosen": best}


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
             "# family log_n variant bucket   (family 0 = fused polymul, 1 = forward, 2 = inverse;",
             "#   bucket = jobs per SM of the launch: 0 <= 1, 1 <= 2, 2 <= 4, 3 more;",
             "#   family 3 log_n 0 = concurrent degree classes, log_n 2 = ragged batches as one launch)"]
    for fam, table in ((POLYMUL, best), (FORWARD, fwd), (INVERSE, inv)):
        lines += [f"{fam} {log_n} {v} {bucket}" for (log_n, bucket), v in sorted(table.items())]
    lines += [f"{BATCH} 0 {1 if conc == 'concurrent' else 0}", f"{BATCH} 2 {1 if conc == 'single_launch' else 0}"]
    with open(out_table, "w") as f:
        f.write("\n".join(lines) + "\n")
    rep = {"gpu_sms": sms, "polymul": report, "forward": fwd_report, "inverse": inv_report,
           "batch_classes": conc_report,
           "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    with open(os.path.splitext(out_table)[0] + "_report.json", "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps({"table": out_table, "polymul": {f"{k[0]}/{k[1]}": v for k, v in best.items()},
                      "forward": {f"{k[0]}/{k[1]}": v for k, v in fwd.items()},
                      "inverse": {f"{k[0]}/{k[1]}": v for k, v in inv.items()}, "ragged_batches": conc}))


if __name__ == "__main__":
    main(sys.argv[1:])
