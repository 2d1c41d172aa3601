"""Failure paths, injected on the host.

Device allocations are made to fail by the library's host-side injector
(vkhel_debug_fail_allocations) -- no GPU fault is involved.  Every entry point
must report the failure as a status (or a NULL object), leave the context
usable, and give correct results once allocations succeed again; a server
fails only the micro-batch whose allocation failed.  Queued server requests
can be cancelled.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

OOM, BUDGET, CANCELLED = 2, 3, 7


@pytest.fixture(autouse=True)
def _injector_off(vk):
    yield
    vk.fail_allocations(0, 0)


def _operands(n, seed=0):
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    rng = np.random.default_rng(seed)
    return q, w, workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)


def test_vector_creation_failure_is_reported_and_recovers(vk, ctx):
    before = ctx.bytes_in_use
    vk.fail_allocations(0, 1)
    with pytest.raises(vk.VkhelError) as e:
        vk.Vector(ctx, 1024)
    assert e.value.code == OOM
    assert ctx.bytes_in_use == before
    v = vk.Vector(ctx, np.arange(1024, dtype=np.uint64))
    np.testing.assert_array_equal(v.download(), np.arange(1024, dtype=np.uint64))


def test_polymul_scratch_failure_then_success(vk, ctx, oracle):
    n = 1 << 12
    q, w, a_h, b_h = _operands(n)
    t = vk.NttTables(n, q, w)
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    vk.polymul(a, b, c, t)              # tables resident; no scratch needed for a separate result
    vk.fail_allocations(0, 1)           # result aliases a: the call needs a scratch buffer
    with pytest.raises(vk.VkhelError) as e:
        vk.polymul(a, b, a, t)
    assert e.value.code == OOM
    np.testing.assert_array_equal(a.download(), a_h)   # nothing ran
    vk.polymul(a, b, a, t)
    np.testing.assert_array_equal(a.download(), oracle.polymul(a_h, b_h, n, q, w)[0])


def test_batch_commit_failure_then_fresh_batch(vk, ctx, oracle):
    n = 1 << 14
    q, w, a_h, b_h = _operands(n, 1)
    t = vk.NttTables(n, q, w)
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    bt = vk.Batch(ctx)
    bt.add_polymul([t], a, b, c)
    vk.fail_allocations(0, 1)           # the device job table
    with pytest.raises(vk.VkhelError) as e:
        bt.commit()
    assert e.value.code == OOM
    bt.close()
    bt = vk.Batch(ctx)
    bt.add_polymul([t], a, b, c)
    bt.commit()
    bt.run()
    np.testing.assert_array_equal(c.download(), oracle.polymul(a_h, b_h, n, q, w)[0])


def test_failed_batch_add_records_nothing(vk, oracle):
    """An add whose second limb's tables cannot be made resident fails as a
    whole: the batch keeps none of that call's jobs, and the same add then
    succeeds and computes the right words."""
    n = 1 << 12
    qs = workloads.ntt_primes(n, 2)
    tabs = [vk.NttTables(n, q, workloads.root_for(n, q)) for q in qs]
    rng = np.random.default_rng(5)
    a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
    b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
    with vk.Context() as fresh:
        a, b, c = vk.Vector(fresh, a_h), vk.Vector(fresh, b_h), vk.Vector(fresh, 2 * n)
        bt = vk.Batch(fresh)
        vk.fail_allocations(1, 1)           # limb 0's tables upload, limb 1's fail
        with pytest.raises(vk.VkhelError) as e:
            bt.add_polymul(tabs, a, b, c)
        assert e.value.code == OOM
        assert bt.jobs == 0
        bt.add_polymul(tabs, a, b, c)
        assert bt.jobs == 2
        bt.commit()
        bt.run()
        got = c.download()
        for k, q in enumerate(qs):
            w = workloads.root_for(n, q)
            want = oracle.polymul(a_h[k * n:(k + 1) * n], b_h[k * n:(k + 1) * n], n, q, w)[0]
            np.testing.assert_array_equal(got[k * n:(k + 1) * n], want)
        bt.close()


def test_batch_commit_retried_after_a_failure(vk, oracle):
    """A commit that fails part-way (here the single-launch item table, after
    the job table was allocated) leaves the batch uncommitted; committing it
    again succeeds, computes the right words and frees everything the first
    attempt had taken."""
    L = vk.lib()
    saved = L.vkhel_tune_get(3, 2)
    L.vkhel_tune_set(3, 2, 1)
    try:
        with vk.Context() as fresh:
            shapes = [(1 << 12, 1), (1 << 14, 2)]
            tabs, vecs, refs = [], [], []
            for n, k in shapes:
                q, w, a_h, b_h = _operands(n, k)
                t = vk.NttTables(n, q, w)
                a, b, c = vk.Vector(fresh, a_h), vk.Vector(fresh, b_h), vk.Vector(fresh, n)
                tabs.append(t)
                vecs.append((a, b, c))
                refs.append(oracle.polymul(a_h, b_h, n, q, w)[0])
            bt = vk.Batch(fresh)
            for t, (a, b, c) in zip(tabs, vecs):
                bt.add_polymul([t], a, b, c)
            before = fresh.bytes_in_use     # the adds made the tables resident
            vk.fail_allocations(1, 1)       # the job table succeeds, the item table fails
            with pytest.raises(vk.VkhelError) as e:
                bt.commit(graph=True)
            assert e.value.code == OOM
            bt.commit(graph=True)
            bt.run()
            assert bt.kernels == 1
            for (a, b, c), ref in zip(vecs, refs):
                np.testing.assert_array_equal(c.download(), ref)
            bt.close()
            fresh.sync()
            assert fresh.bytes_in_use == before
    finally:
        vk.fail_allocations(0, 0)
        L.vkhel_tune_set(3, 2, saved)


def test_elem_batch_commit_retried_after_a_failure(vk, oracle):
    """An element-wise batch whose unit-table allocation fails commits on the
    second try, computes the oracle's words and frees what it took."""
    q = workloads.ntt_primes(1 << 10, 1)[0]
    rng = np.random.default_rng(9)
    with vk.Context() as fresh:
        a_h, b_h = workloads.uniform(rng, q, 5000), workloads.uniform(rng, q, 5000)
        a, b, r = vk.Vector(fresh, a_h), vk.Vector(fresh, b_h), vk.Vector(fresh, 5000)
        before = fresh.bytes_in_use
        eb = vk.ElemBatch(fresh)
        eb.add("elemmul", a, b, r, q)
        vk.fail_allocations(0, 1)
        with pytest.raises(vk.VkhelError) as e:
            eb.commit()
        assert e.value.code == OOM
        eb.commit()
        eb.run()
        np.testing.assert_array_equal(r.download(), oracle.elemmul(a_h, b_h, q))
        eb.close()
        fresh.sync()
        assert fresh.bytes_in_use == before


def test_table_upload_failure_then_success(vk, oracle):
    n = 1 << 10
    q, w, a_h, _ = _operands(n, 2)
    t = vk.NttTables(n, q, w)
    with vk.Context() as fresh:         # no tables resident yet
        a, r = vk.Vector(fresh, a_h), vk.Vector(fresh, n)
        vk.fail_allocations(0, 1)       # the context's first use of (n, q, w): its device tables
        with pytest.raises(vk.VkhelError):
            vk.forward_transform(a, r, t)
        vk.forward_transform(a, r, t)
        np.testing.assert_array_equal(r.download(), oracle.forward(a_h, n, q, w)[0])


def test_budget_exhaustion(vk, ctx):
    ctx.set_budget(ctx.bytes_in_use + 8 * 1024)
    try:
        vk.Vector(ctx, 512)
        with pytest.raises(vk.VkhelError) as e:
            vk.Vector(ctx, 4096)
        assert e.value.code == BUDGET
    finally:
        ctx.set_budget(0)


def test_server_fails_only_the_failing_micro_batch(vk, oracle):
    n = 1 << 13
    q, w, a_h, b_h = _operands(n, 3)
    t = vk.NttTables(n, q, w)
    ref = oracle.polymul(a_h, b_h, n, q, w)[0]
    with vk.Server(max_batch_limbs=4) as srv:
        srv.wait(srv.submit([t], a_h, b_h, np.zeros(n, np.uint64)))   # warm-up: tables resident
        c1 = np.zeros(n, np.uint64)
        vk.fail_allocations(0, 1)
        assert srv.wait(srv.submit([t], a_h, b_h, c1)) == OOM
        c2 = np.zeros(n, np.uint64)
        assert srv.wait(srv.submit([t], a_h, b_h, c2)) == 0
        np.testing.assert_array_equal(c2, ref)
        assert srv.stats()["failed"] >= 1


def test_server_allocation_failure_after_a_chunk_was_issued(vk, oracle):
    """A micro-batch pipelined in limb chunks whose second request's buffer
    cannot be allocated: its first chunk is already uploading and computing.
    The micro-batch's requests fail with OOM (the first may have completed in
    a micro-batch of its own, then correctly), its buffers are released only
    after the issued work, and the server stays usable and exact."""
    n = 1 << 16
    qs = workloads.ntt_primes(n, 8)
    ws = [workloads.root_for(n, q) for q in qs]
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    rng = np.random.default_rng(12)

    def req(limbs):
        a = np.concatenate([workloads.uniform(rng, q, n) for q in qs[:limbs]])
        b = np.concatenate([workloads.uniform(rng, q, n) for q in qs[:limbs]])
        return tabs[:limbs], a, b, np.zeros(limbs * n, np.uint64)

    def check(r):
        t, a, b, c = r
        for k in range(len(t)):
            s = slice(k * n, (k + 1) * n)
            np.testing.assert_array_equal(c[s], oracle.polymul(a[s], b[s], n, qs[k], ws[k])[0])

    blocker, first, second, after = req(8), req(6), req(4), req(8)
    with vk.Server(max_batch_limbs=16, max_inflight_batches=1) as srv:
        assert srv.wait(srv.submit(*req(8))) == 0        # warm-up: tables resident
        vk.fail_allocations(2, 1)                          # the blocker's and the first's succeed
        ids = [srv.submit(*r) for r in (blocker, first, second)]
        st = [srv.wait(i) for i in ids]
        assert st[0] == 0 and st[2] == OOM and st[1] in (0, OOM)
        vk.fail_allocations(0, 0)
        assert srv.wait(srv.submit(*after)) == 0
    check(blocker)
    check(after)
    if st[1] == 0:
        check(first)


def test_server_cancel_queued_request(vk, oracle):
    n = 1 << 16
    q, w, a_h, b_h = _operands(n, 4)
    t = vk.NttTables(n, q, w)
    limbs = 8
    a = np.tile(a_h, limbs)
    b = np.tile(b_h, limbs)
    per = 3 * limbs * n * 8
    # one request at a time (budget), many queued: the last is still queued when cancelled
    with vk.Server(device_budget=per, max_batch_limbs=limbs, max_inflight_batches=1) as srv:
        outs = [np.zeros(limbs * n, np.uint64) for _ in range(12)]
        ids = [srv.submit([t] * limbs, a, b, o) for o in outs]
        st = srv.cancel(ids[-1])
        results = [srv.wait(i) for i in ids]
        assert all(r == 0 for r in results[:-1])
        if st == 0:
            assert results[-1] == CANCELLED
        else:  # it had already started: it must then have completed normally
            assert results[-1] == 0
        assert srv.cancel(ids[0]) != 0      # collected: cannot be cancelled
    ref = oracle.polymul(a_h, b_h, n, q, w)[0]
    np.testing.assert_array_equal(outs[0][:n], ref)
