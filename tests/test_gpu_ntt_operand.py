"""Products with one operand already in the transform domain.

vkhel_vector_polymul_ntt and vkhel_batch_add_polymul_ntt take b as NTT(b),
the words vkhel_vector_forward_transform writes, and compute what the
reference's caller computes with a stored transform: forward(a), then
elemmul(NTT(a), NTT(b)), then inverse (src/vector.c:388-427, 513-657).  With
NTT(b) from the forward transform the result is the negacyclic product of a
and b, so it is checked against the oracle's polymul; with arbitrary 64-bit
words in place of NTT(b) (elemmul reduces its operands) against the oracle's
composition of the same three steps.  Degrees cover the CTA kernels, the
cluster kernels, the split single-call clusters and the composed paths
(n < 2^8, n >= 2^18); moduli both kernel families.  Tolerance zero.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


def _setup(n, bits, seed):
    q = workloads.ntt_primes(n, 1, bound=1 << bits)[0]
    w = workloads.root_for(n, q)
    rng = np.random.default_rng(seed)
    return q, w, workloads.uniform(rng, q, n), workloads.uniform(rng, q, n), rng


@pytest.mark.parametrize("bits", [31, 60, 62, 63])
@pytest.mark.parametrize("log_n", [1, 5, 8, 11, 12, 13, 14, 15, 16, 17, 18, 20])
def test_polymul_ntt_equals_polymul(vk, ctx, oracle, log_n, bits):
    n = 1 << log_n
    if bits < log_n + 8:
        pytest.skip("no NTT prime of this size")
    q, w, a_h, b_h, _ = _setup(n, bits, 100 + log_n)
    t = vk.NttTables(n, q, w)
    if bits == 63 and ((t.arrays()["roots"] >= q).any() or (t.arrays()["inv_roots"] >= q).any()):
        pytest.skip("a table entry not below q: refused by design")
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    bn = vk.Vector(ctx, n)
    vk.forward_transform(b, bn, t)
    vk.polymul_ntt(a, bn, c, t)
    want, st = oracle.polymul(a_h, b_h, n, q, w)
    assert st == 0
    np.testing.assert_array_equal(c.download(), want, err_msg=f"n={n} q={q}")
    np.testing.assert_array_equal(bn.download(), oracle.forward(b_h, n, q, w)[0])  # NTT(b) untouched
    vk.polymul_ntt(a, bn, a, t)  # the result may overwrite a
    np.testing.assert_array_equal(a.download(), want)


@pytest.mark.parametrize("bits", [60, 63])
@pytest.mark.parametrize("log_n", [4, 10, 14, 16, 19])
def test_unreduced_transform_domain_words_follow_elemmul(vk, ctx, oracle, log_n, bits):
    """Any 64-bit words in place of NTT(b): reduced as the reference's
    elemmul reduces its operands, then the inverse transform."""
    n = 1 << log_n
    q, w, a_h, _, rng = _setup(n, bits, 200 + log_n)
    t = vk.NttTables(n, q, w)
    if bits == 63 and ((t.arrays()["roots"] >= q).any() or (t.arrays()["inv_roots"] >= q).any()):
        pytest.skip("a table entry not below q: refused by design")
    bn_h = rng.integers(0, 1 << 64, size=n, dtype=np.uint64)
    bn_h[: n // 2] %= np.uint64(q)  # half canonical, half not
    a, bn, c = vk.Vector(ctx, a_h), vk.Vector(ctx, bn_h), vk.Vector(ctx, n)
    vk.polymul_ntt(a, bn, c, t)
    fa, st = oracle.forward(a_h, n, q, w)
    assert st == 0
    want, st = oracle.inverse(oracle.elemmul(fa, bn_h, q), n, q, w)
    assert st == 0
    np.testing.assert_array_equal(c.download(), want)
    bt = vk.Batch(ctx)
    c2 = vk.Vector(ctx, n)
    bt.add_polymul([t], a, bn, c2, b_ntt=True)
    bt.commit()
    bt.run()
    np.testing.assert_array_equal(c2.download(), want)
    bt.close()


def test_polymul_ntt_rejects_result_aliasing_the_operand(vk, ctx):
    n = 1 << 12
    q = workloads.ntt_primes(n, 1)[0]
    t = vk.NttTables(n, q, workloads.root_for(n, q))
    a, bn = vk.Vector(ctx, n), vk.Vector(ctx, n)
    with pytest.raises(vk.VkhelError) as e:
        vk.polymul_ntt(a, bn, bn, t)
    assert e.value.code == 1 and "aliases" in e.value.msg
    bt = vk.Batch(ctx)
    with pytest.raises(vk.VkhelError) as e:
        bt.add_polymul([t], a, bn, bn, b_ntt=True)
    assert e.value.code == 1 and "overlaps" in e.value.msg
    assert bt.jobs == 0
    bt.close()


@pytest.mark.parametrize("single_launch", [0, 1])
@pytest.mark.parametrize("graph", [True, False])
def test_batch_mixes_transform_domain_and_plain_products(vk, oracle, graph, single_launch):
    """One batch with plain and NTT(b) products of the same and of different
    degrees (fused CTA and cluster classes, composed classes), 60- and 63-bit
    limbs; with the ragged single launch asked for, the NTT(b) classes keep
    the batch on per-class launches and every word is still right."""
    L = vk.lib()
    saved = L.vkhel_tune_get(3, 2)
    L.vkhel_tune_set(3, 2, single_launch)
    try:
        with vk.Context() as c:
            bt = vk.Batch(c)
            checks = []
            shapes = [(6, 60, 2, True), (12, 60, 3, True), (12, 60, 2, False), (14, 63, 2, True),
                      (15, 60, 1, True), (16, 60, 2, False), (16, 60, 1, True), (18, 60, 1, True)]
            for i, (log_n, bits, limbs, pre) in enumerate(shapes):
                n = 1 << log_n
                qs = workloads.ntt_primes(n, limbs, bound=1 << bits)
                ws = [workloads.root_for(n, q) for q in qs]
                tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
                rng = np.random.default_rng(300 + i)
                a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
                b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
                a, b, out = vk.Vector(c, a_h), vk.Vector(c, b_h), vk.Vector(c, limbs * n)
                if pre:  # NTT(b) of every limb, from the oracle's forward transform
                    bn = vk.Vector(c, np.concatenate([oracle.forward(b_h[k * n:(k + 1) * n], n, qs[k], ws[k])[0]
                                                      for k in range(limbs)]))
                    bt.add_polymul(tabs, a, bn, out, b_ntt=True)
                else:
                    bt.add_polymul(tabs, a, b, out)
                want = np.concatenate([oracle.polymul(a_h[k * n:(k + 1) * n], b_h[k * n:(k + 1) * n], n, qs[k],
                                                      ws[k])[0] for k in range(limbs)])
                checks.append((out, want, log_n))
            bt.commit(graph=graph)
            for _ in range(2):
                bt.run()
                for out, want, log_n in checks:
                    np.testing.assert_array_equal(out.download(), want, err_msg=f"log_n={log_n}")
            bt.close()
    finally:
        L.vkhel_tune_set(3, 2, saved)
