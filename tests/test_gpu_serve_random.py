"""Seeded random serving: plain requests and requests on resident operands of
random degree (2^1 .. 2^18), limb count (1 .. 5) and modulus size (30 to 63
bits), submitted from two threads into servers of random micro-batch size
and depth.  Every result must equal the oracle's polymul bit for bit.
"""
import threading

import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


def _tables(vk, n, limbs, bits):
    out = []
    for q in workloads.ntt_primes(n, limbs, bound=1 << bits):
        w = workloads.root_for(n, q)
        t = vk.NttTables(n, q, w)
        ar = t.arrays()
        if (ar["roots"] >= q).any() or (ar["inv_roots"] >= q).any():
            return None  # refused by design
        out.append((q, w, t))
    return out


def _shape(rng):
    log_n = int(rng.integers(1, 19))
    bits = 63 if rng.random() < 0.3 else int(rng.integers(max(30, log_n + 8), 62))
    return 1 << log_n, int(rng.integers(1, 6)), bits


@pytest.mark.parametrize("seed", range(3))
def test_random_requests_match_oracle(vk, oracle, seed):
    rng = np.random.default_rng(500 + seed)
    with vk.Server(max_batch_limbs=int(rng.choice([16, 64, 512])),
                   max_inflight_batches=int(rng.integers(1, 5))) as srv:
        ops = []
        for _ in range(3):
            n, limbs, bits = _shape(rng)
            tl = _tables(vk, n, limbs, bits)
            if tl is None:
                continue
            b = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tl])
            ops.append((tl, b, srv.add_operand([t for _, _, t in tl], b), n))
        items = []
        while len(items) < 40:
            if ops and rng.random() < 0.5:
                tl, b, oid, n = ops[int(rng.integers(0, len(ops)))]
            else:
                n, limbs, bits = _shape(rng)
                tl = _tables(vk, n, limbs, bits)
                if tl is None:
                    continue
                b, oid = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tl]), None
            a = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tl])
            items.append((tl, a, b, np.zeros_like(a), oid, n))
        ids = [None] * len(items)

        def submitter(lo, hi):
            for i in range(lo, hi):
                tl, a, b, c, oid, _ = items[i]
                ts = [t for _, _, t in tl]
                ids[i] = srv.submit_operand(ts, a, oid, c) if oid else srv.submit(ts, a, b, c)

        half = len(items) // 2
        threads = [threading.Thread(target=submitter, args=(0, half)),
                   threading.Thread(target=submitter, args=(half, len(items)))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for (tl, a, b, c, oid, n), rid in zip(items, ids):
            assert srv.wait(rid) == 0
            for k, (q, w, _) in enumerate(tl):
                ref, st = oracle.polymul(a[k * n:(k + 1) * n], b[k * n:(k + 1) * n], n, q, w)
                assert st == 0
                np.testing.assert_array_equal(c[k * n:(k + 1) * n], ref,
                                              err_msg=f"seed {seed} n={n} limb {k} operand={bool(oid)}")
        for _, _, oid, _ in ops:
            srv.remove_operand(oid)
