"""Seeded random call sequences on one context, checked against a shadow copy.

Four vectors of n words and one table set; each step is a random call of
the public API -- forward / inverse transform, polymul, polymul with b in the
transform domain, elemmul, elemgtadd, elemmod, a blocking or asynchronous
upload, copy_from_host, a blocking or asynchronous download, map, sync --
with random operands (results may alias an operand), while stream-ordered
calls (vkhel_ctx_set_async) are switched on and off at random.  The shadow
copy applies the oracle's restatement of each call in program order; every
read-back must equal it bit for bit, whatever was still queued when the
read was issued.  Degrees 2^12 (one CTA), 2^14 and 2^16 (single calls split
over clusters) and 2^18 (passes over HBM).
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

NVEC = 4


def _run_sequence(vk, oracle, log_n, seed, steps=90):
    n = 1 << log_n
    rng = np.random.default_rng(seed)
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    ot = oracle.tables(n, q, w)
    fwd = lambda x: oracle.forward(x, n, q, w, tables=ot)[0]
    inv = lambda x: oracle.inverse(x, n, q, w, tables=ot)[0]
    with vk.Context() as ctx:
        t = vk.NttTables(n, q, w)
        shadow = [workloads.uniform(rng, q, n) for _ in range(NVEC)]
        vecs = [vk.Vector(ctx, s) for s in shadow]
        keep = []      # host buffers of queued async copies
        pending = []   # (host buffer, expected words) of async downloads
        log = []

        def check(i, got, what):
            np.testing.assert_array_equal(got, shadow[i], err_msg=f"seed {seed} n={n} {what} v{i} after {log[-8:]}")

        for step in range(steps):
            op = rng.choice(["fwd", "inv", "mul", "mul_ntt", "elemmul", "gtadd", "mod", "upload", "upload_async",
                             "copy_from_host", "download", "download_async", "map", "sync", "async"],
                            p=[.11, .11, .11, .07, .08, .07, .06, .06, .06, .03, .06, .06, .04, .03, .05])
            a, b, d = (int(x) for x in rng.integers(0, NVEC, size=3))
            log.append(f"{op}({a},{b}->{d})")
            if op == "fwd":
                vk.forward_transform(vecs[a], vecs[d], t)
                shadow[d] = fwd(shadow[a])
            elif op == "inv":
                vk.inverse_transform(vecs[a], vecs[d], t)
                shadow[d] = inv(shadow[a])
            elif op == "mul":
                vk.polymul(vecs[a], vecs[b], vecs[d], t)
                shadow[d] = oracle.polymul(shadow[a], shadow[b], n, q, w)[0]
            elif op == "mul_ntt":
                if d == b:  # the result may not alias NTT(b)
                    d = (b + 1) % NVEC
                vk.polymul_ntt(vecs[a], vecs[b], vecs[d], t)
                shadow[d] = inv(oracle.elemmul(fwd(shadow[a]), shadow[b], q))
            elif op == "elemmul":
                vk.elemmul(vecs[a], vecs[b], vecs[d], q)
                shadow[d] = oracle.elemmul(shadow[a], shadow[b], q)
            elif op == "gtadd":
                bound, diff = q // 2, int(rng.integers(1, 1 << 40))
                vk.elemgtadd(vecs[a], vecs[d], bound, diff)
                shadow[d] = oracle.elemgtadd(shadow[a], bound, diff)
            elif op == "mod":
                vk.elemmod(vecs[a], vecs[d], 65537, q)
                shadow[d] = oracle.elemmod(shadow[a], 65537, q)
            elif op in ("upload", "upload_async", "copy_from_host"):
                h = workloads.uniform(rng, q, n)
                if op == "upload":
                    vecs[d].upload(h)
                elif op == "copy_from_host":
                    vecs[d].copy_from_host(h)
                else:
                    keep.append(h)
                    vecs[d].upload_async(h)
                shadow[d] = h.copy()
            elif op == "download":
                check(d, vecs[d].download(), "download")
            elif op == "download_async":
                buf = np.empty(n, np.uint64)
                keep.append(buf)
                vecs[d].download_async(buf)
                pending.append((buf, shadow[d].copy(), d))
            elif op == "map":
                check(d, vecs[d].map_read(), "map")
            elif op == "sync":
                ctx.sync()
                for buf, want, i in pending:
                    np.testing.assert_array_equal(buf, want, err_msg=f"seed {seed} n={n} download_async v{i}")
                pending.clear()
                keep.clear()
            else:
                ctx.set_async(bool(rng.integers(0, 2)))
        ctx.sync()
        for buf, want, i in pending:
            np.testing.assert_array_equal(buf, want, err_msg=f"seed {seed} n={n} download_async v{i} (end)")
        ctx.set_async(False)
        for i in range(NVEC):
            check(i, vecs[i].download(), "final")


@pytest.mark.parametrize("log_n", [12, 14, 16, 18])
@pytest.mark.parametrize("seed", range(5))
def test_random_call_sequence_matches_shadow(vk, oracle, log_n, seed):
    _run_sequence(vk, oracle, log_n, 9000 + 10 * log_n + seed)
