"""Resident operands of the serving loop (vkhel_server_add_operand /
submit_operand / remove_operand).

A polynomial many requests multiply by is uploaded once -- as b, transformed
on the device, or as NTT(b) from the oracle's forward transform -- and
requests then bring only a.  Each result must equal the oracle's polymul of
a and b bit for bit, alone and mixed with plain requests of other and of the
same degrees (fused CTA and cluster kernels, the composed paths n < 2^8 and
n >= 2^18, 60- and 63-bit limbs).  Mismatched tables, unknown operands and
removal while requests still read an operand are refused; an injected
allocation failure fails the upload alone, or the one request whose buffer
it was, which then no longer holds the operand.
"""
import threading

import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


def _limbs(vk, log_n, limbs, bits=60):
    n = 1 << log_n
    qs = workloads.ntt_primes(n, limbs, bound=1 << bits)
    return [(q, workloads.root_for(n, q), vk.NttTables(n, q, workloads.root_for(n, q))) for q in qs]


def _poly(rng, tq, n):
    return np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tq])


def _check(oracle, tq, a, b, c, what=""):
    n = a.size // len(tq)
    for k, (q, w, _) in enumerate(tq):
        ref, st = oracle.polymul(a[k * n:(k + 1) * n], b[k * n:(k + 1) * n], n, q, w)
        assert st == 0
        np.testing.assert_array_equal(c[k * n:(k + 1) * n], ref, err_msg=f"{what} limb {k} n={n}")


@pytest.mark.parametrize("is_ntt", [False, True])
def test_requests_on_resident_operands_match_oracle(vk, oracle, is_ntt):
    rng = np.random.default_rng(31 + is_ntt)
    shapes = [(6, 2, 60), (12, 3, 60), (14, 2, 63), (16, 1, 60), (17, 2, 60), (18, 1, 60)]
    with vk.Server(max_batch_limbs=16, max_inflight_batches=3) as srv:
        ops = []
        for log_n, limbs, bits in shapes:
            n = 1 << log_n
            tq = _limbs(vk, log_n, limbs, bits)
            b = _poly(rng, tq, n)
            up = b
            if is_ntt:  # NTT(b) of every limb, from the oracle
                up = np.concatenate([oracle.forward(b[k * n:(k + 1) * n], n, q, w)[0] for k, (q, w, _) in enumerate(tq)])
            oid = srv.add_operand([t for _, _, t in tq], up, is_ntt=is_ntt)
            ops.append((tq, b, oid, n))
        pending = []
        for rep in range(3):  # several requests per operand, interleaved with plain ones
            for tq, b, oid, n in ops:
                a = _poly(rng, tq, n)
                c = np.zeros_like(a)
                pending.append((tq, a, b, c, srv.submit_operand([t for _, _, t in tq], a, oid, c), "operand"))
                a2, b2 = _poly(rng, tq, n), _poly(rng, tq, n)
                c2 = np.zeros_like(a2)
                pending.append((tq, a2, b2, c2, srv.submit([t for _, _, t in tq], a2, b2, c2), "plain"))
        for tq, a, b, c, rid, what in pending:
            assert srv.wait(rid) == 0
            _check(oracle, tq, a, b, c, what)
        for _, _, oid, _ in ops:
            srv.remove_operand(oid)


def test_operand_requests_from_threads(vk, oracle):
    rng = np.random.default_rng(41)
    tq = _limbs(vk, 13, 4)
    n = 1 << 13
    b = _poly(rng, tq, n)
    reqs = [(_poly(rng, tq, n), np.zeros(4 * n, np.uint64)) for _ in range(24)]
    with vk.Server(max_batch_limbs=32) as srv:
        oid = srv.add_operand([t for _, _, t in tq], b)
        ids = [None] * len(reqs)

        def submitter(lo, hi):
            for i in range(lo, hi):
                ids[i] = srv.submit_operand([t for _, _, t in tq], reqs[i][0], oid, reqs[i][1])

        threads = [threading.Thread(target=submitter, args=(i, i + 8)) for i in range(0, len(reqs), 8)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for (a, c), rid in zip(reqs, ids):
            assert srv.wait(rid) == 0
            _check(oracle, tq, a, b, c)
        stats = srv.stats()
        assert stats["completed"] == len(reqs) and stats["failed"] == 0


def test_operand_misuse_is_refused(vk, oracle):
    rng = np.random.default_rng(51)
    tq = _limbs(vk, 12, 2)
    n = 1 << 12
    with vk.Server() as srv:
        oid = srv.add_operand([t for _, _, t in tq], _poly(rng, tq, n))
        a, c = _poly(rng, tq, n), np.zeros(2 * n, np.uint64)
        with pytest.raises(vk.VkhelError) as e:  # other primes
            srv.submit_operand([t for _, _, t in _limbs(vk, 12, 2, bits=59)], a, oid, c)
        assert e.value.code == 1 and "differ" in e.value.msg
        with pytest.raises(vk.VkhelError) as e:  # one limb fewer
            srv.submit_operand([tq[0][2]], a[:n], oid, c[:n])
        assert e.value.code == 1
        with pytest.raises(vk.VkhelError) as e:
            srv.submit_operand([t for _, _, t in tq], a, oid + 5, c)
        assert e.value.code == 1 and "unknown" in e.value.msg
        # removal while a queued or running request reads the operand
        rid = srv.submit_operand([t for _, _, t in tq], a, oid, c)
        try:
            srv.remove_operand(oid)
            removed_early = True
        except vk.VkhelError as err:
            assert err.code == 1 and "read by" in err.msg
            removed_early = False
        assert srv.wait(rid) == 0
        if not removed_early:
            srv.remove_operand(oid)
        with pytest.raises(vk.VkhelError):
            srv.remove_operand(oid)
        with pytest.raises(vk.VkhelError):
            srv.submit_operand([t for _, _, t in tq], a, oid, c)


def test_operand_upload_failure_is_reported_and_the_server_goes_on(vk, oracle):
    rng = np.random.default_rng(61)
    tq = _limbs(vk, 14, 2)
    n = 1 << 14
    b = _poly(rng, tq, n)
    with vk.Server() as srv:
        vk.fail_allocations(0, 1)
        try:
            with pytest.raises(vk.VkhelError) as e:
                srv.add_operand([t for _, _, t in tq], b)
            assert e.value.code == 2
        finally:
            vk.fail_allocations(0, 0)
        oid = srv.add_operand([t for _, _, t in tq], b)
        a, c = _poly(rng, tq, n), np.zeros(2 * n, np.uint64)
        assert srv.wait(srv.submit_operand([t for _, _, t in tq], a, oid, c)) == 0
        _check(oracle, tq, a, b, c)


def test_failed_request_releases_its_operand(vk, oracle):
    """A request on a resident operand whose buffer allocation fails reports
    out-of-memory; the operand is then read by nobody and can be removed, and
    the next request on it succeeds."""
    rng = np.random.default_rng(71)
    tq = _limbs(vk, 12, 2)
    n = 1 << 12
    b = _poly(rng, tq, n)
    with vk.Server() as srv:
        oid = srv.add_operand([t for _, _, t in tq], b)
        a, c = _poly(rng, tq, n), np.zeros(2 * n, np.uint64)
        vk.fail_allocations(0, 1)
        try:
            assert srv.wait(srv.submit_operand([t for _, _, t in tq], a, oid, c)) == 2
        finally:
            vk.fail_allocations(0, 0)
        assert srv.wait(srv.submit_operand([t for _, _, t in tq], a, oid, c)) == 0
        _check(oracle, tq, a, b, c)
        srv.remove_operand(oid)
        assert srv.stats()["failed"] == 1
