"""Serving loop (vkhel_server_*): continuous batching of polymul requests.

Requests of mixed degree (2^4 .. 2^17) and limb count are submitted from
several threads while earlier ones run; every result must equal the oracle's
reference composition bit for bit -- the same as the request computed alone.
Admission under a device budget smaller than the offered load, waits with a
timeout, and error reporting are exercised too.
"""
import threading

import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

_PRIMES = {}


def _tables(vk, log_n, limbs):
    n = 1 << log_n
    if n not in _PRIMES:
        qs = workloads.ntt_primes(n, 6)
        _PRIMES[n] = [(q, workloads.root_for(n, q), vk.NttTables(n, q, workloads.root_for(n, q))) for q in qs]
    return _PRIMES[n][:limbs]


def _request(vk, rng, log_n, limbs):
    n = 1 << log_n
    tq = _tables(vk, log_n, limbs)
    a = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tq])
    b = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tq])
    c = np.zeros(limbs * n, np.uint64)
    return tq, a, b, c


def _check(oracle, tq, a, b, c):
    n = a.size // len(tq)
    for k, (q, w, _) in enumerate(tq):
        ref, st = oracle.polymul(a[k * n:(k + 1) * n], b[k * n:(k + 1) * n], n, q, w)
        assert st == 0
        np.testing.assert_array_equal(c[k * n:(k + 1) * n], ref, err_msg=f"limb {k} n={n}")


def test_mixed_requests_from_threads_match_alone(vk, oracle):
    rng = np.random.default_rng(21)
    shapes = [(4, 1), (9, 2), (12, 3), (13, 1), (14, 4), (15, 2), (16, 1), (17, 1), (12, 6), (10, 5)] * 3
    reqs = [_request(vk, rng, l, k) for l, k in shapes]
    with vk.Server(max_batch_limbs=16, max_inflight_batches=3) as srv:
        ids = [None] * len(reqs)

        def submitter(lo, hi):
            for i in range(lo, hi):
                tq, a, b, c = reqs[i]
                ids[i] = srv.submit([t for _, _, t in tq], a, b, c)

        threads = [threading.Thread(target=submitter, args=(i, i + 10)) for i in range(0, len(reqs), 10)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for rid in ids:
            assert srv.wait(rid) == 0
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["batches"] < len(reqs)  # requests shared micro-batches
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    for tq, a, b, c in reqs:
        _check(oracle, tq, a, b, c)
    # the same requests alone, one server call each, give the same words
    with vk.Server() as srv:
        for tq, a, b, c in reqs[:10]:
            alone = np.zeros_like(c)
            assert srv.wait(srv.submit([t for _, _, t in tq], a, b, alone)) == 0
            np.testing.assert_array_equal(alone, c)


def test_large_micro_batches_run_in_limb_chunks(vk, oracle):
    """At low load, micro-batches of at most four requests and 8 MB of
    operands or more are issued in up to four chunks of limbs (each computing
    as soon as its operands are up).  First the requests go in small groups,
    each after the previous group finished: the 12.6 MB request alone runs in
    three chunks (boundaries inside the request); 6.3 + 3.1 MB, when the
    scheduler takes the pair together, in two (a boundary between requests).
    Then all at once, while the first micro-batch runs: the next one takes
    every queued request that fits and may be chunked too."""
    rng = np.random.default_rng(41)
    shapes = [(17, 6), (16, 5), (14, 6), (17, 3), (15, 6), (16, 4)]
    reqs = [_request(vk, rng, l, k) for l, k in shapes]
    with vk.Server(max_batch_limbs=20, max_inflight_batches=1) as srv:
        for pair in ((0,), (1, 2), (3, 4), (5,)):
            for rid in [srv.submit([t for _, _, t in reqs[i][0]], *reqs[i][1:]) for i in pair]:
                assert srv.wait(rid) == 0
        for tq, a, b, c in reqs:
            _check(oracle, tq, a, b, c)
            c[:] = 0
        ids = [srv.submit([t for _, _, t in tq], a, b, c) for tq, a, b, c in reqs]
        for rid in ids:
            assert srv.wait(rid) == 0
        assert srv.stats()["completed"] == 2 * len(reqs)
    for tq, a, b, c in reqs:
        _check(oracle, tq, a, b, c)


def test_admission_under_a_small_budget(vk, oracle):
    rng = np.random.default_rng(5)
    reqs = [_request(vk, rng, 14, 2) for _ in range(12)]
    per_req = 3 * 2 * (1 << 14) * 8
    with vk.Server(device_budget=2 * per_req, max_batch_limbs=64) as srv:
        ids = [srv.submit([t for _, _, t in tq], a, b, c) for tq, a, b, c in reqs]
        for rid in ids:
            assert srv.wait(rid) == 0
        assert srv.stats()["batches"] >= 6  # at most two requests fit at a time
    for tq, a, b, c in reqs:
        _check(oracle, tq, a, b, c)


def test_wait_timeout_and_bad_requests(vk):
    rng = np.random.default_rng(8)
    with vk.Server(max_batch_limbs=8) as srv:
        tq, a, b, c = _request(vk, rng, 17, 8)
        rid = srv.submit([t for _, _, t in tq], a, b, c)
        st = srv.wait(rid, timeout_ms=0)
        assert st in (0, 6)  # finished already or still running
        if st == 6:
            assert srv.wait(rid) == 0
        with pytest.raises(vk.VkhelError):
            srv.submit([t for _, _, t in tq] * 2, np.zeros(16 * (1 << 17), np.uint64),
                       np.zeros(16 * (1 << 17), np.uint64), np.zeros(16 * (1 << 17), np.uint64))
        assert srv.wait(12345) == 1  # unknown id
