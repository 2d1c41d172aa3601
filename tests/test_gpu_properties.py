"""Size-independent properties at the benchmark's full sizes.

The oracle checks small and medium sizes word for word; at the headline
batch (n = 16384, 8 limbs of 60-bit primes, 32 pairs = 256 limb products,
seed 2) and at the largest degrees these algebraic identities must hold
exactly, computed entirely by the library:
  * commutativity      a * b = b * a
  * distributivity     a * (b + d) = a * b + a * d   (additions by elemfma_canonical)
  * linearity          NTT(x + y) = NTT(x) + NTT(y)  (n = 2^17, 2^18)
and one limb of each product is compared with the oracle as an anchor.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

N, LIMBS, PAIRS, SEED = 16384, 8, 32, 2


def _batch_products(vk, ctx, tabs, a, b, out):
    bt = vk.Batch(ctx)
    stride = LIMBS * N
    for i in range(PAIRS):
        bt.add_polymul(tabs, a.device_ptr + 8 * i * stride, b.device_ptr + 8 * i * stride,
                       out.device_ptr + 8 * i * stride)
    bt.commit(graph=True)
    bt.run()
    bt.close()


def _add_limbwise(vk, ctx, x, y, qs, words_per_limb, total_limbs):
    """x + y mod q of each limb (limb k of every pair uses qs[k % LIMBS])."""
    out = vk.Vector(ctx, x.length)
    eb = vk.ElemBatch(ctx)
    for l in range(total_limbs):
        off = 8 * l * words_per_limb
        eb.add("elemfma_canonical", x.device_ptr + off, y.device_ptr + off,
               (out.device_ptr + off, words_per_limb), 1, qs[l % len(qs)])
    eb.commit(graph=False)
    eb.run()
    eb.close()
    return out


def test_headline_batch_commutes_and_distributes(vk, ctx, oracle):
    qs, ws, a_h, b_h = workloads.rns_batch(N, LIMBS, PAIRS, SEED)
    _, _, d_h, _ = workloads.rns_batch(N, LIMBS, PAIRS, SEED + 100)
    tabs = [vk.NttTables(N, q, w) for q, w in zip(qs, ws)]
    a, b, d = vk.Vector(ctx, a_h.ravel()), vk.Vector(ctx, b_h.ravel()), vk.Vector(ctx, d_h.ravel())
    words = PAIRS * LIMBS * N
    ab, ba, ad = vk.Vector(ctx, words), vk.Vector(ctx, words), vk.Vector(ctx, words)
    _batch_products(vk, ctx, tabs, a, b, ab)
    _batch_products(vk, ctx, tabs, b, a, ba)
    _batch_products(vk, ctx, tabs, a, d, ad)
    bd = _add_limbwise(vk, ctx, b, d, qs, N, PAIRS * LIMBS)
    a_bd = vk.Vector(ctx, words)
    _batch_products(vk, ctx, tabs, a, bd, a_bd)
    ab_ad = _add_limbwise(vk, ctx, ab, ad, qs, N, PAIRS * LIMBS)
    got_ab = ab.download()
    np.testing.assert_array_equal(got_ab, ba.download(), err_msg="a * b != b * a")
    np.testing.assert_array_equal(a_bd.download(), ab_ad.download(), err_msg="a * (b + d) != a * b + a * d")
    # anchor: the last pair's limb 7 against the oracle
    ref, _ = oracle.polymul(a_h[-1, 7], b_h[-1, 7], N, qs[7], ws[7])
    np.testing.assert_array_equal(got_ab[-N:], ref)


@pytest.mark.parametrize("log_n", [17, 18])
def test_forward_transform_is_linear_at_the_largest_degrees(vk, ctx, oracle, log_n):
    n = 1 << log_n
    limbs = 4
    qs = workloads.ntt_primes(n, limbs)
    ws = [workloads.root_for(n, q) for q in qs]
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    rng = np.random.default_rng(log_n)
    x_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
    y_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
    x, y = vk.Vector(ctx, x_h), vk.Vector(ctx, y_h)
    xy = _add_limbwise(vk, ctx, x, y, qs, n, limbs)
    fx, fy, fxy = (vk.Vector(ctx, limbs * n) for _ in range(3))
    bt = vk.Batch(ctx)
    bt.add_transform(tabs, x, fx)
    bt.add_transform(tabs, y, fy)
    bt.add_transform(tabs, xy, fxy)
    bt.commit(graph=True)
    bt.run()
    bt.close()
    sum_f = _add_limbwise(vk, ctx, fx, fy, qs, n, limbs)
    np.testing.assert_array_equal(fxy.download(), sum_f.download(), err_msg="NTT(x + y) != NTT(x) + NTT(y)")
    np.testing.assert_array_equal(fx.download(n), oracle.forward(x_h[:n], n, qs[0], ws[0])[0])
