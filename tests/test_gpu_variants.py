"""Every compiled kernel variant is bit-exact (with and without an epilogue).

The autotuner only chooses among variants (words per thread, radix-16 groups
in flight per thread, concurrent degree classes), so each variant of each
family must give the oracle's words for every degree it exists for.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

VARIANTS = {8: [0, 1], 9: [0, 1], 10: [0, 1, 2], 11: [0, 1, 2], 12: [0, 1, 2], 13: [0, 1, 2], 14: [0, 1]}


@pytest.mark.parametrize("log_n", sorted(VARIANTS))
def test_every_variant_matches_oracle(vk, ctx, oracle, log_n):
    L = vk.lib()
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(log_n + 500)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    a_h[1] = (1 << 64) - 1  # exact first-stage path
    ref_poly, _ = oracle.polymul(a_h, b_h, n, q, w)
    ref_lift = oracle.elemgtadd(oracle.elemmod(ref_poly, 65537, q), q // 3, 5)
    ref_fwd, _ = oracle.forward(a_h, n, q, w)
    saved = [L.vkhel_tune_get(f, log_n) for f in range(3)]
    split = L.vkhel_tune_get(3, 1)
    L.vkhel_tune_set(3, 1, 1)  # single calls on one CTA (not split over a cluster): the variants run
    try:
        for v in VARIANTS[log_n]:
            for f in range(3):
                L.vkhel_tune_set(f, log_n, v)
            a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
            vk.polymul(a, b, c, t)
            np.testing.assert_array_equal(c.download(), ref_poly, err_msg=f"polymul variant {v}")
            vk.polymul_lift(a, b, c, t, [("elemmod", 65537, 0), ("elemgtadd", q // 3, 5)])
            np.testing.assert_array_equal(c.download(), ref_lift, err_msg=f"lifted polymul variant {v}")
            vk.forward_transform(a, c, t)
            np.testing.assert_array_equal(c.download(), ref_fwd, err_msg=f"forward variant {v}")
            vk.inverse_transform(c, c, t)
            np.testing.assert_array_equal(c.download(), oracle.inverse(ref_fwd, n, q, w)[0],
                                          err_msg=f"inverse variant {v}")
    finally:
        for f in range(3):
            L.vkhel_tune_set(f, log_n, saved[f])
        L.vkhel_tune_set(3, 1, split)


@pytest.mark.parametrize("log_n", [12, 13, 14, 15, 16])
@pytest.mark.parametrize("split", [0, 1, 2])
def test_single_calls_split_or_not_are_exact(vk, ctx, oracle, log_n, split):
    """A single call of n = 2^12 .. 2^16 runs on a cluster -- 16 CTAs with
    2^10 .. 2^12-word sub-blocks from n = 2^14 (split = 0), 8 CTAs with 2^9 ..
    2^13-word ones below or with tuning entry (3, 3) = 1 (split = 2) -- unless
    the split is switched off (split = 1); all give the oracle's words."""
    L = vk.lib()
    saved16 = L.vkhel_tune_get(3, 3)
    L.vkhel_tune_set(3, 3, 1 if split == 2 else 0)
    split = 1 if split == 1 else 0
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1, bound=1 << 62)[0]
    w = workloads.root_for(n, q)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(log_n + 40 * split)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    a_h[3] = (1 << 64) - 1  # exact first-stage rule
    saved = L.vkhel_tune_get(3, 1)
    try:
        L.vkhel_tune_set(3, 1, split)
        a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
        vk.polymul(a, b, c, t)
        np.testing.assert_array_equal(c.download(), oracle.polymul(a_h, b_h, n, q, w)[0])
        vk.polymul_lift(a, b, c, t, [("elemmod", 2, 0)])
        np.testing.assert_array_equal(c.download(), oracle.elemmod(oracle.polymul(a_h, b_h, n, q, w)[0], 2, q))
        vk.forward_transform(a, c, t)
        np.testing.assert_array_equal(c.download(), oracle.forward(a_h, n, q, w)[0])
        x = c.download()
        # unreduced first operand of a first-stage pair (the reference's
        # subtraction loop is defined for it; a second operand this large
        # would make that loop wrap, which the oracle reports)
        x[4] = (1 << 64) - 3
        c.upload(x)
        vk.inverse_transform(c, c, t)
        ref, st = oracle.inverse(x, n, q, w)
        assert st == 0
        np.testing.assert_array_equal(c.download(), ref)
    finally:
        L.vkhel_tune_set(3, 1, saved)
        L.vkhel_tune_set(3, 3, saved16)


@pytest.mark.parametrize("concurrent", [0, 1])
def test_batch_class_concurrency_is_exact(vk, ctx, oracle, concurrent):
    L = vk.lib()
    saved = L.vkhel_tune_get(3, 0)
    rng = np.random.default_rng(77 + concurrent)
    cases = []
    try:
        L.vkhel_tune_set(3, 0, concurrent)
        bt = vk.Batch(ctx)
        for log_n, limbs in [(12, 2), (13, 1), (14, 3), (15, 1), (16, 1), (9, 2), (6, 1)]:
            n = 1 << log_n
            qs = workloads.ntt_primes(n, limbs)
            ws = [workloads.root_for(n, q) for q in qs]
            tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
            a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
            b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
            va, vb, vc = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, limbs * n)
            bt.add_polymul(tabs, va, vb, vc)
            cases.append((qs, ws, a_h, b_h, vc, n, tabs, va, vb))
        bt.commit(graph=True)
        bt.run()
        bt.run()
    finally:
        L.vkhel_tune_set(3, 0, saved)
    for qs, ws, a_h, b_h, vc, n, *_ in cases:
        got = vc.download()
        for k, (q, w) in enumerate(zip(qs, ws)):
            ref, _ = oracle.polymul(a_h[k * n:(k + 1) * n], b_h[k * n:(k + 1) * n], n, q, w)
            np.testing.assert_array_equal(got[k * n:(k + 1) * n], ref)
