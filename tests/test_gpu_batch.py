"""Batched polynomial multiply (vkhel_batch_*) against the oracle.

Covers equal-degree RNS batches in one fused launch, ragged batches mixing
degrees (fused classes and composed classes for n < 256 and n > 2^14),
results aliasing an operand, CUDA-graph replay picking up new operand data,
and the eager (non-graph) path.  Every limb product must equal the
reference composition forward, forward, elemmul, inverse bit for bit.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


def _check(oracle, qs, ws, a_h, b_h, c_h, n):
    for k, (q, w) in enumerate(zip(qs, ws)):
        ref, st = oracle.polymul(a_h[k * n:(k + 1) * n], b_h[k * n:(k + 1) * n], n, q, w)
        assert st == 0
        np.testing.assert_array_equal(c_h[k * n:(k + 1) * n], ref, err_msg=f"limb {k}")


@pytest.mark.parametrize("graph", [True, False])
def test_rns_batch(vk, ctx, oracle, graph):
    n, limbs, pairs = 4096, 3, 5
    qs, ws, a, b = workloads.rns_batch(n, limbs, pairs, seed=9)
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    batch = vk.Batch(ctx)
    vecs = []
    for i in range(pairs):
        va, vb = vk.Vector(ctx, a[i].ravel()), vk.Vector(ctx, b[i].ravel())
        vc = vk.Vector(ctx, limbs * n)
        batch.add_polymul(tabs, va, vb, vc)
        vecs.append((va, vb, vc))
    batch.commit(graph=graph)  # runs nothing
    assert batch.jobs == pairs * limbs
    assert all(not vc.download().any() for _, _, vc in vecs)
    before = vk.launch_count()
    batch.run()
    assert batch.kernels >= 1 and vk.launch_count() - before == batch.kernels
    for i, (va, vb, vc) in enumerate(vecs):
        _check(oracle, qs, ws, a[i].ravel(), b[i].ravel(), vc.download(), n)
    # new operand data in the same vectors is picked up by the next launch
    rng = np.random.default_rng(77)
    a2 = np.stack([workloads.uniform(rng, q, n) for q in qs]).ravel()
    vecs[0][0].upload(a2)
    batch.run()
    _check(oracle, qs, ws, a2, b[0].ravel(), vecs[0][2].download(), n)


def test_ragged_batch_mixes_degrees_and_aliasing(vk, ctx, oracle):
    rng = np.random.default_rng(5)
    batch = vk.Batch(ctx)
    cases = []
    for log_n, limbs, alias in [(4, 2, False), (9, 1, True), (12, 3, False), (14, 2, True), (15, 1, False),
                                (13, 2, False), (12, 1, True), (16, 1, True), (7, 4, False)]:
        n = 1 << log_n
        qs = workloads.ntt_primes(n, limbs)
        ws = [workloads.root_for(n, q) for q in qs]
        tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
        a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        va, vb = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h)
        vc = va if alias else vk.Vector(ctx, limbs * n)
        batch.add_polymul(tabs, va, vb, vc)
        cases.append((qs, ws, a_h, b_h, vc, n, tabs, va, vb))
    batch.commit(graph=True)
    batch.run()
    for qs, ws, a_h, b_h, vc, n, *_ in cases:
        _check(oracle, qs, ws, a_h, b_h, vc.download(), n)


@pytest.mark.parametrize("graph", [True, False])
def test_scratch_slices_after_tiny_products_stay_aligned(vk, oracle, graph):
    """Products of n = 2 (3 limbs) need NTT(b) scratch slices of 2 words each;
    the slices of the larger products after them (n = 2^18 composed, n = 2^14
    with c aliasing a) must still start on 32-byte boundaries, where their
    kernels move 16 words at a time with 32-byte vector accesses."""
    rng = np.random.default_rng(88)
    with vk.Context() as c:
        batch = vk.Batch(c)
        cases = []
        # unpadded, the slices of n = 2 and 4 (3 limbs each) would end 144 bytes in
        for log_n, limbs, alias in [(1, 3, False), (18, 2, False), (14, 2, True), (2, 3, True)]:
            n = 1 << log_n
            qs = workloads.ntt_primes(n, limbs)
            ws = [workloads.root_for(n, q) for q in qs]
            tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
            a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
            b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
            va, vb = vk.Vector(c, a_h), vk.Vector(c, b_h)
            vc = va if alias else vk.Vector(c, limbs * n)
            batch.add_polymul(tabs, va, vb, vc)
            cases.append((qs, ws, a_h, b_h, vc, n, tabs, va, vb))
        batch.commit(graph=graph)
        batch.run()
        for qs, ws, a_h, b_h, vc, n, *_ in cases:
            _check(oracle, qs, ws, a_h, b_h, vc.download(), n)
        batch.close()


def test_batch_raw_device_pointers(vk, ctx, oracle):
    n, limbs = 8192, 2
    qs, ws, a, b = workloads.rns_batch(n, limbs, 1, seed=4)
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    va, vb, vc = vk.Vector(ctx, a[0].ravel()), vk.Vector(ctx, b[0].ravel()), vk.Vector(ctx, limbs * n)
    batch = vk.Batch(ctx)
    batch.add_polymul(tabs, va.device_ptr, vb.device_ptr, vc.device_ptr)
    batch.commit(graph=True)
    batch.run()
    _check(oracle, qs, ws, a[0].ravel(), b[0].ravel(), vc.download(), n)


def test_batch_rejects_bad_input(vk, ctx):
    n = 1024
    q = workloads.ntt_primes(n, 1)[0]
    t = vk.NttTables(n, q, workloads.root_for(n, q))
    batch = vk.Batch(ctx)
    short = vk.Vector(ctx, n - 1)
    ok = vk.Vector(ctx, n)
    with pytest.raises(vk.VkhelError):
        batch.add_polymul([t], short, ok, ok)
    with pytest.raises(vk.VkhelError):
        batch.commit()  # empty
    with pytest.raises(vk.VkhelError):
        batch.launch()  # not committed


@pytest.mark.parametrize("graph", [True, False])
def test_batch_transforms_mixed_with_polymul(vk, ctx, oracle, graph):
    """Forward and inverse transforms (in place and not, an inverse with a lift)
    and polymuls of several degrees in one batch equal the oracle."""
    rng = np.random.default_rng(31 + graph)
    bt = vk.Batch(ctx)
    checks = []
    for log_n, limbs in [(2, 2), (8, 3), (12, 2), (14, 4), (15, 1), (16, 2), (18, 1), (13, 40)]:
        n = 1 << log_n
        qs = workloads.ntt_primes(n, limbs) if log_n > 2 else [113, 17][:limbs]
        ws = [workloads.root_for(n, q) for q in qs]
        tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
        x_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        y_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        x, y = vk.Vector(ctx, x_h), vk.Vector(ctx, y_h)
        fwd_out = vk.Vector(ctx, limbs * n)
        bt.add_transform(tabs, x, fwd_out)                                   # forward, out of place
        bt.add_transform(tabs, y, y, inverse=True)                           # inverse, in place
        lifted = vk.Vector(ctx, limbs * n)
        bt.add_transform(tabs, x, lifted, inverse=True, lift=[("elemmod", 65537, 0)])
        prod = vk.Vector(ctx, limbs * n)
        bt.add_polymul(tabs, x, vk.Vector(ctx, y_h), prod)
        checks.append((n, qs, ws, x_h, y_h, fwd_out, y, lifted, prod))
    bt.commit(graph=graph)
    bt.run()
    for n, qs, ws, x_h, y_h, fwd_out, y, lifted, prod in checks:
        f, i, l, p = fwd_out.download(), y.download(), lifted.download(), prod.download()
        for k, (q, w) in enumerate(zip(qs, ws)):
            s = slice(k * n, (k + 1) * n)
            np.testing.assert_array_equal(f[s], oracle.forward(x_h[s], n, q, w)[0], err_msg=f"forward n={n}")
            np.testing.assert_array_equal(i[s], oracle.inverse(y_h[s], n, q, w)[0], err_msg=f"inverse n={n}")
            np.testing.assert_array_equal(l[s], oracle.elemmod(oracle.inverse(x_h[s], n, q, w)[0], 65537, q),
                                          err_msg=f"lifted inverse n={n}")
            np.testing.assert_array_equal(p[s], oracle.polymul(x_h[s], y_h[s], n, q, w)[0], err_msg=f"polymul n={n}")


def test_batch_transform_rejects_bad_arguments(vk, ctx):
    n = 1024
    q = workloads.ntt_primes(n, 1)[0]
    t = vk.NttTables(n, q, workloads.root_for(n, q))
    x, y = vk.Vector(ctx, n), vk.Vector(ctx, n // 2)
    bt = vk.Batch(ctx)
    with pytest.raises(vk.VkhelError):
        bt.add_transform([t], x, y)                                          # output too short
    with pytest.raises(vk.VkhelError):
        bt.add_transform([t], x, x, inverse=False, lift=[("elemmod", 3, 0)])  # lift on a forward


@pytest.mark.parametrize("log_n", [6, 10, 14, 15, 17])
def test_polymul_result_may_alias_the_second_operand(vk, ctx, oracle, log_n):
    """c = b (the fused kernels park NTT(b) in c): single call and batch."""
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(log_n + 300)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    ref, _ = oracle.polymul(a_h, b_h, n, q, w)
    a, b = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h)
    vk.polymul(a, b, b, t)
    np.testing.assert_array_equal(b.download(), ref, err_msg="single call")
    jobs = 24  # enough jobs that the batch takes the one-CTA / cluster-per-job paths
    a2 = vk.Vector(ctx, np.tile(a_h, jobs))
    b2 = vk.Vector(ctx, np.tile(b_h, jobs))
    bt = vk.Batch(ctx)
    bt.add_polymul([t] * jobs, a2, b2, b2)
    bt.commit(graph=True)
    bt.run()
    np.testing.assert_array_equal(b2.download(), np.tile(ref, jobs), err_msg="batch")
