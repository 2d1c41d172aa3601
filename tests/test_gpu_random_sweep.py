"""A seeded sweep over the parameter space the reference accepts.

Each case draws a degree n = 2^k (k in 1..18), a modulus size of 20 to 63
bits (63 in about a third of the cases), one of the first NTT primes of that size and a random primitive 2n-th
root w (not only the smallest one, so that the 63-bit tables whose
reference-built "powers" wrap appear with other roots too), and inputs that
are partly unreduced.  The forward and inverse transforms, the fused or
composed product and the batch path must equal the oracle bit for bit.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

def _case(seed):
    rng = np.random.default_rng(seed)
    log_n = int(rng.integers(1, 19))
    n = 1 << log_n
    bits = 63 if rng.random() < 0.3 else int(rng.integers(20, 63))  # the top range often
    bits = max(bits, log_n + 8)
    qs = workloads.ntt_primes(n, 3, bound=1 << bits)
    q = qs[int(rng.integers(0, len(qs)))]
    w0 = workloads.root_for(n, q)
    w = pow(w0, 2 * int(rng.integers(0, n)) + 1, q)  # every primitive 2n-th root is an odd power of one
    a = workloads.uniform(rng, q, n)
    b = workloads.uniform(rng, q, n)
    k = min(n, 4)
    a[:k] = rng.integers(0, 1 << 62, size=k, dtype=np.uint64)  # unreduced words below 2^62
    return n, q, w, a, b


@pytest.mark.parametrize("seed", range(40))
def test_random_parameters_match_oracle(vk, ctx, oracle, seed):
    n, q, w, a_h, b_h = _case(seed)
    t = vk.NttTables(n, q, w)
    if (t.arrays()["roots"] >= q).any() or (t.arrays()["inv_roots"] >= q).any():
        pytest.skip("a table entry not below q: refused by design")
    ot = oracle.tables(n, q, w)
    a, b, r = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    vk.forward_transform(a, r, t)
    f_ref, st = oracle.forward(a_h, n, q, w, ot)
    assert st == 0
    np.testing.assert_array_equal(r.download(), f_ref, err_msg=f"forward n={n} q={q} w={w}")
    vk.inverse_transform(a, r, t)
    i_ref, st = oracle.inverse(a_h, n, q, w, ot)
    assert st == 0
    np.testing.assert_array_equal(r.download(), i_ref, err_msg=f"inverse n={n} q={q} w={w}")
    vk.polymul(a, b, r, t)
    p_ref, st = oracle.polymul(a_h, b_h, n, q, w)
    assert st == 0
    np.testing.assert_array_equal(r.download(), p_ref, err_msg=f"polymul n={n} q={q} w={w}")
    bt = vk.Batch(ctx)
    c = vk.Vector(ctx, n)
    bt.add_polymul([t], a, b, c)
    bt.commit(graph=True)
    bt.run()
    bt.close()
    np.testing.assert_array_equal(c.download(), p_ref, err_msg=f"batch n={n} q={q} w={w}")
