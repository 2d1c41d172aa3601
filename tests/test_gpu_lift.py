"""Centred-lift epilogues fused after the inverse transform.

vkhel_vector_polymul_lift / vkhel_vector_inverse_transform_lift /
vkhel_batch_add_polymul_lift must equal the unfused composition: the
transform, then the reference's elemmod / elemgtsub / elemgtadd one after
another on the result (here the oracle's restatement of each), for every
size class (simple kernels, one CTA, one cluster, the multi-pass 2^18 path).
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def _apply(oracle, x, steps, q):
    for st in steps:
        if st[0] == "elemmod":
            x = oracle.elemmod(x, st[1], st[2] or q)
        elif st[0] == "elemgtsub":
            x = oracle.elemgtsub(x, st[1], st[2], st[3])
        else:
            x = oracle.elemgtadd(x, st[1], st[2])
    return x


def _chains(q):
    return [
        [("elemmod", 65537, 0)],                                   # BFV-style centred reduction mod t
        [("elemmod", 2, q)],                                       # centred parity
        [("elemgtsub", q // 2, q, 1 << 40), ("elemgtadd", q // 3, M64 - 5)],   # wrap in gtadd
        [("elemgtadd", q // 2, (1 << 62) - q), ("elemmod", 3, 0), ("elemgtsub", 1, 5, 3),
         ("elemmod", (1 << 63) + 29, 1 << 62)],                    # four steps, 64-bit modulus
    ]


@pytest.mark.parametrize("log_n", [2, 6, 8, 11, 13, 14, 15, 16, 17, 18])
def test_polymul_lift_matches_composition(vk, ctx, oracle, log_n):
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(900 + log_n)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    ref, _ = oracle.polymul(a_h, b_h, n, q, w)
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    for steps in _chains(q):
        vk.polymul_lift(a, b, c, t, steps)
        np.testing.assert_array_equal(c.download(), _apply(oracle, ref, steps, q), err_msg=str(steps))
    vk.polymul(a, b, c, t)  # no epilogue afterwards: plain product again
    np.testing.assert_array_equal(c.download(), ref)


@pytest.mark.parametrize("log_n", [0, 3, 9, 14, 15, 17, 18])
def test_inverse_lift_covers_whole_result(vk, ctx, oracle, log_n):
    n = 1 << log_n
    q = workloads.ntt_primes(max(n, 2), 1, bound=1 << 50)[0]
    w = workloads.root_for(max(n, 2), q) if n > 1 else 3
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(40 + log_n)
    extra = 37
    a_h = workloads.uniform(rng, q, n)
    tail = workloads.uniform(rng, q, extra)
    res_h = np.concatenate([np.zeros(n, np.uint64), tail])
    # reference: inverse over n words (none at n = 1: the result is left as
    # it was), n^-1 scaling of the words past them, then the ops on all words
    ref = res_h.copy()
    start = n if n > 1 else 0
    if n > 1:
        ref[:n] = oracle.inverse(a_h, n, q, w)[0]
    ninv = pow(n, -1, q)
    ref[start:] = np.array([(int(x) * ninv) % q for x in res_h[start:]], dtype=np.uint64)
    a = vk.Vector(ctx, a_h)
    for steps in _chains(q):
        res = vk.Vector(ctx, res_h)
        vk.inverse_transform_lift(a, res, t, steps)
        np.testing.assert_array_equal(res.download(), _apply(oracle, ref, steps, q), err_msg=str(steps))


def test_batch_lifts_per_add_and_per_limb_modulus(vk, ctx, oracle):
    rng = np.random.default_rng(5)
    bt = vk.Batch(ctx)
    cases = []
    chains = [None, [("elemmod", 65537, 0)], [("elemmod", 2, 0), ("elemgtadd", 0, 7)],
              [("elemgtsub", 1 << 58, 3, 1 << 20)]]
    for i, (log_n, limbs) in enumerate([(12, 3), (12, 2), (12, 1), (13, 2), (16, 2), (6, 2), (6, 1), (18, 1),
                                        (12, 2), (16, 1)]):
        n = 1 << log_n
        qs = workloads.ntt_primes(n, limbs)
        ws = [workloads.root_for(n, q) for q in qs]
        tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
        a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        va, vb, vc = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, limbs * n)
        steps = chains[i % len(chains)]
        bt.add_polymul(tabs, va, vb, vc, lift=steps)
        cases.append((qs, ws, a_h, b_h, vc, n, steps, tabs, va, vb))
    bt.commit(graph=True)
    bt.run()
    bt.run()
    for qs, ws, a_h, b_h, vc, n, steps, *_ in cases:
        got = vc.download()
        for k, (q, w) in enumerate(zip(qs, ws)):
            ref, _ = oracle.polymul(a_h[k * n:(k + 1) * n], b_h[k * n:(k + 1) * n], n, q, w)
            if steps:
                ref = _apply(oracle, ref, steps, q)
            np.testing.assert_array_equal(got[k * n:(k + 1) * n], ref, err_msg=f"n={n} limb {k} {steps}")


def test_lift_rejects_bad_steps(vk, ctx):
    n = 1024
    q = workloads.ntt_primes(n, 1)[0]
    t = vk.NttTables(n, q, workloads.root_for(n, q))
    a, b, c = vk.Vector(ctx, n), vk.Vector(ctx, n), vk.Vector(ctx, n)
    for steps in ([("elemmod", 7, 0)] * 5, [("elemmod", 1, q)], [("elemgtsub", 1, 1, 0)], [(9, 1, 1, 1)]):
        with pytest.raises(vk.VkhelError):
            vk.polymul_lift(a, b, c, t, steps)


@pytest.mark.parametrize("log_n,jobs", [(1, 300), (5, 257), (7, 64), (11, 40), (18, 3)])
def test_batched_inverse_lift_of_many_jobs(vk, ctx, oracle, log_n, jobs):
    """A batch of inverse transforms with a lift on the multi-launch degrees
    (n < 2^8: one block per job in the epilogue pass; 2^18: contiguous block
    ranges across job boundaries) and a fused one (2^11), four primes
    alternating, against the oracle's inverse followed by the ops."""
    n = 1 << log_n
    qs = workloads.ntt_primes(n, 4)
    ws = [workloads.root_for(n, q) for q in qs]
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    rng = np.random.default_rng(700 + log_n)
    x_h = np.concatenate([workloads.uniform(rng, qs[j % 4], n) for j in range(jobs)])
    x, y = vk.Vector(ctx, x_h), vk.Vector(ctx, jobs * n)
    steps = [("elemmod", 65537, 0), ("elemgtadd", 1 << 15, 1 << 40)]
    bt = vk.Batch(ctx)
    bt.add_transform([tabs[j % 4] for j in range(jobs)], x, y, inverse=True, lift=steps)
    bt.commit(graph=True)
    bt.run()
    got = y.download()
    for j in range(jobs):
        q, w = qs[j % 4], ws[j % 4]
        ref = _apply(oracle, oracle.inverse(x_h[j * n:(j + 1) * n], n, q, w)[0], steps, q)
        np.testing.assert_array_equal(got[j * n:(j + 1) * n], ref, err_msg=f"job {j}")
