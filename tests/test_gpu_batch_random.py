"""Seeded random batches: many kinds of job in one committed batch.

Each case draws 4 to 12 adds, each of a random kind -- a product, a product
with b in the transform domain, a forward transform, an inverse transform
with or without a centred-lift epilogue -- of a random degree 2^1 .. 2^19,
1 to 4 limbs of 30- to 63-bit primes, sometimes in place; commits the batch
(graph or eager, the concurrent-class tuning on or off) and launches it
twice, with fresh operands before the second launch.  Every output word must
equal the oracle's: polymul, forward, inverse and the element-wise ops of the
epilogue, limb by limb.  This exercises the class split (kind, degree,
modulus class, epilogue, operand form), the scratch slices and the stream
fork of one commit together.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

KINDS = ("polymul", "polymul_ntt", "forward", "inverse", "inverse_lift")


def _limb_tables(vk, n, limbs, bits, cache):
    key = (n, limbs, bits)
    if key not in cache:
        qs = workloads.ntt_primes(n, limbs, bound=1 << bits)
        ok = []
        for q in qs:
            w = workloads.root_for(n, q)
            t = vk.NttTables(n, q, w)
            ar = t.arrays()
            if bits == 63 and ((ar["roots"] >= q).any() or (ar["inv_roots"] >= q).any()):
                return None  # refused by design
            ok.append((q, w, t))
        cache[key] = ok
    return cache[key]


def _expect(oracle, kind, tl, a, b, n, lift):
    out = []
    for k, (q, w, _) in enumerate(tl):
        x = a[k * n:(k + 1) * n]
        if kind in ("polymul", "polymul_ntt"):
            r, st = oracle.polymul(x, b[k * n:(k + 1) * n], n, q, w)
        elif kind == "forward":
            r, st = oracle.forward(x, n, q, w)
        else:
            r, st = oracle.inverse(x, n, q, w)
            if kind == "inverse_lift":
                r = oracle.elemmod(r, lift, q)
        assert st == 0
        out.append(r)
    return np.concatenate(out)


@pytest.mark.parametrize("seed", range(12))
def test_random_mixed_batch_matches_oracle(vk, oracle, seed):
    rng = np.random.default_rng(7000 + seed)
    graph = bool(seed % 2)
    L = vk.lib()
    saved = L.vkhel_tune_get(3, 0)
    L.vkhel_tune_set(3, 0, int((seed // 2) % 2))  # classes on concurrent streams or in sequence
    cache = {}
    try:
        with vk.Context() as ctx:
            bt = vk.Batch(ctx)
            adds = []
            for _ in range(int(rng.integers(4, 13))):
                kind = KINDS[int(rng.integers(0, len(KINDS)))]
                log_n = int(rng.integers(1, 20))
                n = 1 << log_n
                limbs = int(rng.integers(1, 5))
                bits = 63 if rng.random() < 0.25 else int(rng.integers(max(30, log_n + 8), 63))
                tl = _limb_tables(vk, n, limbs, bits, cache)
                if tl is None:
                    continue
                tabs = [t for _, _, t in tl]
                a_h = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tl])
                b_h = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tl])
                a = vk.Vector(ctx, a_h)
                in_place = kind in ("forward", "inverse", "inverse_lift") and rng.random() < 0.4
                out = a if in_place else vk.Vector(ctx, limbs * n)
                lift = 65537
                b = None
                if kind == "polymul":
                    b = vk.Vector(ctx, b_h)
                    bt.add_polymul(tabs, a, b, out)
                elif kind == "polymul_ntt":
                    bn = np.concatenate([oracle.forward(b_h[k * n:(k + 1) * n], n, q, w)[0]
                                         for k, (q, w, _) in enumerate(tl)])
                    b = vk.Vector(ctx, bn)
                    bt.add_polymul(tabs, a, b, out, b_ntt=True)
                elif kind == "forward":
                    bt.add_transform(tabs, a, out)
                elif kind == "inverse":
                    bt.add_transform(tabs, a, out, inverse=True)
                else:
                    bt.add_transform(tabs, a, out, inverse=True, lift=[("elemmod", lift, 0)])
                adds.append((kind, tl, a, b, out, n, limbs, a_h, b_h, lift))
            bt.commit(graph=graph)
            for launch in range(2):
                if launch == 1:  # fresh operands in the same vectors
                    for i, (kind, tl, a, b, out, n, limbs, _, b_h, lift) in enumerate(adds):
                        a_h = np.concatenate([workloads.uniform(rng, q, n) for q, _, _ in tl])
                        a.upload(a_h)
                        adds[i] = (kind, tl, a, b, out, n, limbs, a_h, b_h, lift)
                bt.run()
                for kind, tl, a, b, out, n, limbs, a_h, b_h, lift in adds:
                    want = _expect(oracle, kind, tl, a_h, b_h, n, lift)
                    np.testing.assert_array_equal(out.download()[:limbs * n], want,
                                                  err_msg=f"seed {seed} launch {launch} {kind} n={n} limbs={limbs}")
            bt.close()
    finally:
        L.vkhel_tune_set(3, 0, saved)
