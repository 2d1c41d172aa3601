"""The benchmark's five workloads, built exactly and compared with the CPU
oracle word for word (tolerance zero: integer arithmetic).

  plain_small        n = 4096, one 60-bit prime, seed 0: forward, inverse
                     round trip, pointwise modmul, polymul (public API calls)
  single_limb_batch  n = 65536, 64 polynomials, seed 1: the 64 products of one
                     batched cluster launch, and the 64 forward / inverse
                     transforms of one batch, plus pointwise mul / add
  rns_batch          n = 16384, 8 primes, 32 pairs, seed 2: all 256 limb
                     products of the fused batch (graph replay), and the same
                     batch fed and drained through the asynchronous copies
  ragged_batch       512 instances, n = 2^12..2^16, 1..16 limbs, seed 3: all
                     4225 limb products of one committed batch
  serving            48 requests of the serving sweep (seed 4, n = 2^12..2^17,
                     1..24 limbs) submitted at once to a server, each also
                     alone: every limb of every result

The oracle follows the reference's stage loops and shader arithmetic
(src/vector.c:513-657, src/kernels/shaders/*.comp); the reference's own test
compares its transforms word for word the same way (test/vector.c:285-329).
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


def _oracle_products(oracle, n, qs, ws, a_rows, b_rows, prime_idx):
    """Oracle limb products of a (count, n) batch with the primes' tables built once."""
    tabs = oracle.batch_tables(n, qs, ws)
    c, _ = oracle.polymul_batch(a_rows, b_rows, n, qs, ws, prime_idx, tables=tabs)
    return c


def test_plain_small_config(vk, ctx, oracle):
    cfg = workloads.CONFIGS["plain_small"]
    n = cfg["n"]
    qs, ws, a_h, b_h = workloads.rns_batch(n, 1, 1, cfg["seed"])
    q, w = qs[0], ws[0]
    a_h, b_h = a_h[0, 0], b_h[0, 0]
    t = vk.NttTables(n, q, w)
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    vk.forward_transform(a, c, t)
    fa = oracle.forward(a_h, n, q, w)[0]
    np.testing.assert_array_equal(c.download(), fa)
    vk.inverse_transform(c, c, t)
    np.testing.assert_array_equal(c.download(), a_h)
    fb = vk.Vector(ctx, n)
    vk.forward_transform(b, fb, t)
    fa_v = vk.Vector(ctx, fa)
    vk.elemmul(fa_v, fb, c, q)
    np.testing.assert_array_equal(c.download(), oracle.elemmul(fa, oracle.forward(b_h, n, q, w)[0], q))
    vk.polymul(a, b, c, t)
    ref, st = oracle.polymul(a_h, b_h, n, q, w)
    assert st == 0
    np.testing.assert_array_equal(c.download(), ref)
    np.testing.assert_array_equal(ref, oracle.schoolbook(a_h, b_h, n, q))


def test_single_limb_batch_config(vk, ctx, oracle):
    cfg = workloads.CONFIGS["single_limb_batch"]
    n, count = cfg["n"], cfg["pairs"]
    qs, ws, a_h, b_h = workloads.rns_batch(n, 1, count, cfg["seed"])
    q, w = qs[0], ws[0]
    a_h, b_h = a_h[:, 0], b_h[:, 0]
    t = vk.NttTables(n, q, w)
    a, b = vk.Vector(ctx, a_h.ravel()), vk.Vector(ctx, b_h.ravel())
    c = vk.Vector(ctx, count * n)
    bt = vk.Batch(ctx)
    for i in range(count):
        bt.add_polymul([t], a.device_ptr + 8 * i * n, b.device_ptr + 8 * i * n, c.device_ptr + 8 * i * n)
    bt.commit(graph=True)
    bt.run()
    assert bt.kernels == 1
    got = c.download().reshape(count, n)
    ref = _oracle_products(oracle, n, [q], [w], a_h, b_h, np.zeros(count, np.uint32))
    np.testing.assert_array_equal(got, ref)
    bt.close()
    # the transforms of the same 64 vectors, batched, and pointwise mul / add
    fa, fb = vk.Vector(ctx, count * n), vk.Vector(ctx, count * n)
    bt = vk.Batch(ctx)
    bt.add_transform([t] * count, a, fa)
    bt.add_transform([t] * count, b, fb)
    bt.commit(graph=True)
    bt.run()
    bt.close()
    tabs = oracle.tables(n, q, w)
    fa_h, fb_h = fa.download().reshape(count, n), fb.download().reshape(count, n)
    for i in range(count):
        np.testing.assert_array_equal(fa_h[i], oracle.forward(a_h[i], n, q, w, tables=tabs)[0], err_msg=f"fwd {i}")
        np.testing.assert_array_equal(fb_h[i], oracle.forward(b_h[i], n, q, w, tables=tabs)[0], err_msg=f"fwd b {i}")
    prod, summ = vk.Vector(ctx, count * n), vk.Vector(ctx, count * n)
    vk.elemmul(fa, fb, prod, q)
    vk.elemfma_canonical(fa, fb, summ, 1, q)
    np.testing.assert_array_equal(prod.download(), oracle.elemmul(fa_h.ravel(), fb_h.ravel(), q))
    np.testing.assert_array_equal(summ.download(), oracle.elemfma_canonical(fa_h.ravel(), fb_h.ravel(), 1, q))
    back = vk.Vector(ctx, count * n)
    bt = vk.Batch(ctx)
    bt.add_transform([t] * count, prod, back, inverse=True)
    bt.commit(graph=False)
    bt.run()
    bt.close()
    np.testing.assert_array_equal(back.download().reshape(count, n), ref)


def _rns_batch_setup(vk, ctx):
    cfg = workloads.CONFIGS["rns_batch"]
    n, limbs, pairs = cfg["n"], cfg["limbs"], cfg["pairs"]
    qs, ws, a_h, b_h = workloads.rns_batch(n, limbs, pairs, cfg["seed"])
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    return n, limbs, pairs, qs, ws, a_h, b_h, tabs


def _rns_reference(oracle, n, limbs, pairs, qs, ws, a_h, b_h):
    pidx = np.tile(np.arange(limbs, dtype=np.uint32), pairs)
    return _oracle_products(oracle, n, qs, ws, a_h.reshape(-1, n), b_h.reshape(-1, n), pidx)


def test_rns_batch_config_every_limb_product(vk, ctx, oracle):
    n, limbs, pairs, qs, ws, a_h, b_h, tabs = _rns_batch_setup(vk, ctx)
    words, stride = pairs * limbs * n, limbs * n
    a, b, c = vk.Vector(ctx, a_h.ravel()), vk.Vector(ctx, b_h.ravel()), vk.Vector(ctx, words)
    bt = vk.Batch(ctx)
    for i in range(pairs):
        bt.add_polymul(tabs, a.device_ptr + 8 * i * stride, b.device_ptr + 8 * i * stride,
                       c.device_ptr + 8 * i * stride)
    bt.commit(graph=True)
    ref = _rns_reference(oracle, n, limbs, pairs, qs, ws, a_h, b_h)
    for rep in range(2):  # the first graph launch and a replay
        bt.launch()
        ctx.sync()
        np.testing.assert_array_equal(c.download().reshape(-1, n), ref, err_msg=f"launch {rep}")
    bt.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_rns_batch_through_async_copies(vk, oracle, pinned):
    """vkhel_vector_upload_async / download_async around a batch launch (the
    end-to-end path of the benchmark), with pinned and pageable host memory,
    whole and partial counts; vkhel_ctx_sync completes everything."""
    torch = pytest.importorskip("torch")
    with vk.Context() as ctx:
        n, limbs, pairs, qs, ws, a_h, b_h, tabs = _rns_batch_setup(vk, ctx)
        words, stride = pairs * limbs * n, limbs * n

        def host(src=None):
            if pinned:
                t = torch.zeros(words, dtype=torch.int64).pin_memory()
                if src is not None:
                    t.numpy().view(np.uint64)[:] = src
                return t, t.numpy().view(np.uint64)
            arr = np.zeros(words, np.uint64) if src is None else np.ascontiguousarray(src, np.uint64)
            return arr, arr

        (ha, _), (hb, _), (hc, hc_np) = host(a_h.ravel()), host(b_h.ravel()), host()
        a, b, c = vk.Vector(ctx, words), vk.Vector(ctx, words), vk.Vector(ctx, words)
        bt = vk.Batch(ctx)
        for i in range(pairs):
            bt.add_polymul(tabs, a.device_ptr + 8 * i * stride, b.device_ptr + 8 * i * stride,
                           c.device_ptr + 8 * i * stride)
        bt.commit(graph=True)
        ref = _rns_reference(oracle, n, limbs, pairs, qs, ws, a_h, b_h)
        a.upload_async(ha)
        b.upload_async(hb)
        bt.launch()
        c.download_async(hc)
        ctx.sync()
        np.testing.assert_array_equal(hc_np.reshape(-1, n), ref)
        # partial counts: refresh only the first pair's a, read back only it
        _, _, a2, _ = workloads.rns_batch(n, limbs, 1, 99)
        (ha2, _), (hc2, hc2_np) = host(np.concatenate([a2.ravel(), a_h.ravel()[stride:]])), host()
        a.upload_async(ha2, stride)
        bt.launch()
        c.download_async(hc2, stride)
        ctx.sync()
        ref2 = _oracle_products(oracle, n, qs, ws, a2.reshape(-1, n), b_h[0].reshape(-1, n),
                                np.arange(limbs, dtype=np.uint32))
        np.testing.assert_array_equal(hc2_np[:stride].reshape(-1, n), ref2)
        assert not hc2_np[stride:].any(), "download_async wrote past its count"
        with pytest.raises(vk.VkhelError):
            a.upload_async(ha, words + 1)
        bt.close()


def test_ragged_batch_config_every_limb_product(vk, ctx, oracle):
    inst = workloads.ragged_batch(512, seed=3)
    vecs = []
    bt = vk.Batch(ctx)
    tabs = {}
    for n, qs, ws, a_h, b_h in inst:
        for q, w in zip(qs, ws):
            if (n, q) not in tabs:
                tabs[(n, q)] = vk.NttTables(n, q, w)
        va, vb, vc = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, len(qs) * n)
        bt.add_polymul([tabs[(n, q)] for q in qs], va, vb, vc)
        vecs.append(vc)
    bt.commit(graph=True)
    bt.run()
    assert bt.jobs == sum(len(x[1]) for x in inst) == 4225
    bt.close()
    # the oracle per degree: every limb product of that degree in one call
    by_n = {}
    for i, (n, qs, ws, a_h, b_h) in enumerate(inst):
        by_n.setdefault(n, []).append(i)
    for n, idx in by_n.items():
        qs_all, ws_all = inst[max(idx, key=lambda i: len(inst[i][1]))][1:3]
        rows_a = np.concatenate([inst[i][3].reshape(-1, n) for i in idx])
        rows_b = np.concatenate([inst[i][4].reshape(-1, n) for i in idx])
        pidx = np.concatenate([np.arange(len(inst[i][1]), dtype=np.uint32) for i in idx])
        for i in idx:  # every instance of a degree uses a prefix of the same primes
            assert list(inst[i][1]) == list(qs_all[:len(inst[i][1])])
        ref = _oracle_products(oracle, n, qs_all, ws_all, rows_a, rows_b, pidx)
        got = np.concatenate([vecs[i].download().reshape(-1, n) for i in idx])
        np.testing.assert_array_equal(got, ref, err_msg=f"degree {n}")


def test_serving_config_each_result_alone_and_in_the_mix(vk, oracle):
    reqs = workloads.serving_requests(48, seed=4)
    tabs = {}
    for n, qs, ws, _, _ in reqs:
        for q, w in zip(qs, ws):
            if (n, q) not in tabs:
                tabs[(n, q)] = vk.NttTables(n, q, w)
    mix = [np.zeros(len(r[1]) * r[0], np.uint64) for r in reqs]
    alone = [np.zeros_like(m) for m in mix]
    with vk.Server(device_budget=40 << 30) as srv:
        ids = [srv.submit([tabs[(n, q)] for q in qs], a, b, c) for (n, qs, ws, a, b), c in zip(reqs, mix)]
        assert all(srv.wait(r) == 0 for r in ids)
        for (n, qs, ws, a, b), c in zip(reqs, alone):
            assert srv.wait(srv.submit([tabs[(n, q)] for q in qs], a, b, c)) == 0
    for i, (n, qs, ws, a, b) in enumerate(reqs):
        ref = _oracle_products(oracle, n, qs, ws, a.reshape(-1, n), b.reshape(-1, n),
                               np.arange(len(qs), dtype=np.uint32))
        np.testing.assert_array_equal(mix[i].reshape(-1, n), ref, err_msg=f"request {i} in the mix")
        np.testing.assert_array_equal(alone[i], mix[i], err_msg=f"request {i} alone")
