"""Small workloads, one per kernel family, for profiling a kernel alone.

    python -m vkhel_gb300.cases NAME [--reps R]
    python -m vkhel_gb300.cases all

Each case builds its inputs (seeded, uniform mod 60-bit primes unless the
name says otherwise), runs its launch once as a warm-up and then R more
times (default 2), synchronizes and prints one line.  The inputs exceed the
129 MB L2 where the kernel streams from HBM, and stay at a few hundred MB on
the device so that a profiler capture of one launch ends quickly.

  fwd_batch     1024 forward transforms of n = 2^14 (batch)     k_ntt_fwd<14,..>
  inv_batch     1024 inverse transforms of n = 2^14 (batch)     k_ntt_inv<14,..>
  fwd_cluster   64 forward transforms of n = 2^16 (batch)       k_ntt_fwd_cluster<2,..>
  inv_cluster   64 inverse transforms of n = 2^16 (batch)       k_ntt_inv_cluster<2,..>
  twiddles      device twiddle tables for n = 2^20              k_twiddles
  global        16 forward + 16 inverse transforms of n = 2^20  k_fwd_global, k_inv_global
  pointwise     32 polymuls of n = 2^18 (composed path)         k_pointwise
  simple        4096 forward + inverse transforms of n = 2^7    k_ntt_fwd_simple, k_ntt_inv_simple
  wide_polymul  256 polymuls of n = 2^14, 63-bit primes         k_polymul<14,..,Mod63>
  cluster_polymul  64 polymuls of n = 2^16 (single-limb batch)  k_polymul_cluster<2,..>
  ragged_single  256 ragged instances, n = 2^12..2^16, as one launch   k_polymul_ragged
  elementwise   elemgtsub / elemmod / elemgtadd / elemfma / elemmul on 2^25 words   k_elementwise<...>
  elementwise_rest  elemmod mod 2, elemfma_canonical, the n^-1 scaling and lift of
                the words past n of an inverse transform      k_elementwise<...>, k_lift_range
  wide_transforms  1024 forward transforms of n = 2^14 and 64 of n = 2^16, 63-bit primes
                k_ntt_fwd<14,..,Mod63>, k_ntt_fwd_cluster<2, Shape<14,32,1,Mod63>>
  ntt_operand   256 polymuls of n = 2^14 with b given as NTT(b)  k_polymul<14,..,true> (the
                epilogue instantiation, no steps)
  lift_jobs     32 inverse transforms of n = 2^20 with a two-step centred lift
                k_inv_global, k_ntt_inv<14,..>, k_lift_stream (the epilogue pass)
  single_call_n65536  one polymul and one forward transform of n = 2^16 as single calls
                k_polymul_cluster<4, Shape<12,16>>, k_ntt_fwd_cluster<4, ..> (16-CTA clusters)
"""
import argparse
import sys

import numpy as np

import vkhel_gb300 as vk
from vkhel_gb300 import workloads


def _tabs(n, count, bits=60):
    qs = workloads.ntt_primes(n, count, bound=1 << bits)
    return qs, [vk.NttTables(n, q, workloads.root_for(n, q)) for q in qs]


def _operands(ctx, n, qs, jobs, seed):
    rng = np.random.default_rng(seed)
    h = np.concatenate([workloads.uniform(rng, qs[j % len(qs)], n) for j in range(jobs)])
    return vk.Vector(ctx, h)


def _transform_batch(ctx, n, jobs, inverse, primes=8):
    qs, tabs = _tabs(n, primes)
    x = _operands(ctx, n, qs, jobs, n + jobs)
    y = vk.Vector(ctx, jobs * n)
    bt = vk.Batch(ctx)
    bt.add_transform([tabs[j % primes] for j in range(jobs)], x, y, inverse=inverse)
    bt.commit(graph=True)
    return bt.launch, (bt, x, y, tabs)


def _polymul_batch(ctx, n, jobs, bits=60, primes=8):
    qs, tabs = _tabs(n, primes, bits)
    a, b = _operands(ctx, n, qs, jobs, 1), _operands(ctx, n, qs, jobs, 2)
    c = vk.Vector(ctx, jobs * n)
    bt = vk.Batch(ctx)
    for j in range(0, jobs, primes):
        k = min(primes, jobs - j)
        bt.add_polymul(tabs[:k], a.device_ptr + 8 * j * n, b.device_ptr + 8 * j * n, c.device_ptr + 8 * j * n)
    bt.commit(graph=True)
    return bt.launch, (bt, a, b, c, tabs)


def case_fwd_batch(ctx):
    return _transform_batch(ctx, 1 << 14, 1024, False)


def case_inv_batch(ctx):
    return _transform_batch(ctx, 1 << 14, 1024, True)


def case_fwd_cluster(ctx):
    return _transform_batch(ctx, 1 << 16, 64, False)


def case_inv_cluster(ctx):
    return _transform_batch(ctx, 1 << 16, 64, True)


def case_twiddles(ctx):
    n = 1 << 20
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    keep = []

    def run():  # another primitive 2n-th root w^(2k+1) per call: fresh tables, generated on the device
        t = vk.NttTables(n, q, pow(w, 2 * len(keep) + 1, q))
        t.device_arrays(ctx)
        keep.append(t)
    return run, keep


def case_global(ctx):
    n, jobs = 1 << 20, 16
    fwd, kf = _transform_batch(ctx, n, jobs, False, primes=4)
    inv, ki = _transform_batch(ctx, n, jobs, True, primes=4)
    return (lambda: (fwd(), inv())), (kf, ki)


def case_pointwise(ctx):
    return _polymul_batch(ctx, 1 << 18, 32, primes=4)


def case_simple(ctx):
    n, jobs = 1 << 7, 4096
    fwd, kf = _transform_batch(ctx, n, jobs, False)
    inv, ki = _transform_batch(ctx, n, jobs, True)
    return (lambda: (fwd(), inv())), (kf, ki)


def case_wide_polymul(ctx):
    return _polymul_batch(ctx, 1 << 14, 256, bits=63)


def case_cluster_polymul(ctx):
    return _polymul_batch(ctx, 1 << 16, 64, primes=1)


def case_ntt_operand(ctx):
    n, jobs, primes = 1 << 14, 256, 8
    qs, tabs = _tabs(n, primes)
    a, b = _operands(ctx, n, qs, jobs, 1), _operands(ctx, n, qs, jobs, 2)
    bn, c = vk.Vector(ctx, jobs * n), vk.Vector(ctx, jobs * n)
    ft = vk.Batch(ctx)  # NTT(b), once, outside the profiled launches
    ft.add_transform([tabs[j % primes] for j in range(jobs)], b, bn)
    ft.commit(graph=False)
    ft.run()
    ft.close()
    bt = vk.Batch(ctx)
    for j in range(0, jobs, primes):
        bt.add_polymul(tabs, a.device_ptr + 8 * j * n, bn.device_ptr + 8 * j * n, c.device_ptr + 8 * j * n,
                       b_ntt=True)
    bt.commit(graph=True)
    return bt.launch, (bt, a, b, bn, c, tabs)


def case_single_call_n65536(ctx):
    n = 1 << 16
    qs, tabs = _tabs(n, 1)
    a, b = _operands(ctx, n, qs, 1, 1), _operands(ctx, n, qs, 1, 2)
    c = vk.Vector(ctx, n)

    def calls():
        vk.polymul(a, b, c, tabs[0])
        vk.forward_transform(a, c, tabs[0])
    return calls, (a, b, c, tabs)


def case_ragged_single(ctx):
    inst = workloads.ragged_batch(256, seed=33)
    tabs, keep = {}, []
    vk.lib().vkhel_tune_set(3, 2, 1)  # the single-launch form for this process
    bt = vk.Batch(ctx)
    for n, qs, ws, a, b in inst:
        for q, w in zip(qs, ws):
            tabs.setdefault((n, q), vk.NttTables(n, q, w))
        va, vb, vc = vk.Vector(ctx, a), vk.Vector(ctx, b), vk.Vector(ctx, len(qs) * n)
        bt.add_polymul([tabs[(n, q)] for q in qs], va, vb, vc)
        keep.append((va, vb, vc))
    bt.commit(graph=True)
    return bt.launch, (bt, keep, tabs)


def case_elementwise(ctx):
    words = 1 << 25
    q = (1 << 61) - 1
    rng = np.random.default_rng(7)
    a = vk.Vector(ctx, workloads.uniform(rng, q, words))
    b = vk.Vector(ctx, workloads.uniform(rng, q, words))
    r = vk.Vector(ctx, words)

    def run():
        vk.elemgtsub(a, r, q // 2, q, 65537)
        vk.elemmod(a, r, 65537, q)
        vk.elemgtadd(a, r, q // 2, 17)
        vk.elemfma(a, b, r, 12345, q)
        vk.elemmul(a, b, r, q)
    return run, (a, b, r)


def case_elementwise_rest(ctx):
    words = 1 << 25
    q = (1 << 61) - 1
    rng = np.random.default_rng(9)
    a = vk.Vector(ctx, workloads.uniform(rng, q, words))
    b = vk.Vector(ctx, workloads.uniform(rng, q, words))
    r = vk.Vector(ctx, words)
    n = 1 << 14
    qq = workloads.ntt_primes(n, 1)[0]
    t = vk.NttTables(n, qq, workloads.root_for(n, qq))
    long_in = vk.Vector(ctx, workloads.uniform(rng, qq, words))

    def run():
        vk.elemmod(a, r, 2, q)                  # OpModTwo
        vk.elemfma_canonical(a, b, r, 12345, q)  # OpFmaCanon
        # an inverse transform into a vector of 2^25 words: the words past n
        # are scaled by n^-1 (OpMulConst) and lifted (k_lift_range)
        vk.inverse_transform_lift(long_in, r, t, [("elemmod", 65537, 0)])
    return run, (a, b, r, t, long_in)


def case_wide_transforms(ctx):
    f14, k14 = _wide_transform_batch(ctx, 1 << 14, 1024)
    f16, k16 = _wide_transform_batch(ctx, 1 << 16, 64)
    return (lambda: (f14(), f16())), (k14, k16)


def case_lift_jobs(ctx):
    """32 inverse transforms of n = 2^20 (256 MB) with the centred-lift
    epilogue: the global passes leave the words in HBM and k_lift_stream
    applies the steps (elemmod 65537, elemgtadd) as its own element-wise
    pass."""
    n, jobs, primes = 1 << 20, 32, 4
    qs, tabs = _tabs(n, primes)
    x = _operands(ctx, n, qs, jobs, 5)
    y = vk.Vector(ctx, jobs * n)
    bt = vk.Batch(ctx)
    bt.add_transform([tabs[j % primes] for j in range(jobs)], x, y, inverse=True,
                     lift=[("elemmod", 65537, 0), ("elemgtadd", 32768, 1 << 40)])
    bt.commit(graph=True)
    return bt.launch, (bt, x, y, tabs)


def _wide_transform_batch(ctx, n, jobs, primes=8):
    qs, tabs = _tabs(n, primes, bits=63)
    x = _operands(ctx, n, qs, jobs, n + jobs)
    y = vk.Vector(ctx, jobs * n)
    bt = vk.Batch(ctx)
    bt.add_transform([tabs[j % primes] for j in range(jobs)], x, y)
    bt.commit(graph=True)
    return bt.launch, (bt, x, y, tabs)


CASES = {k[5:]: v for k, v in globals().items() if k.startswith("case_")}


def run_case(name, reps=2):
    with vk.Context() as ctx:
        fn, keep = CASES[name](ctx)
        fn()  # warm-up: one-time set-up and first graph launch
        ctx.sync()
        for _ in range(reps):
            fn()
        ctx.sync()
        del keep
    print(f"case {name}: {reps} launches after one warm-up", flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("name", choices=sorted(CASES) + ["all"])
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args(argv)
    for name in sorted(CASES) if args.name == "all" else [args.name]:
        run_case(name, args.reps)


if __name__ == "__main__":
    sys.exit(main())
