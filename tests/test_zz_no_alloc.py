"""vkhel_vector_polymul_noalloc: the polynomial multiply for callers that
cannot let the library allocate device memory where they multiply (their
device memory is all held by their own allocator or a fixed reservation, or
a latency-critical loop must not call cudaMalloc / cudaFree, which can wait
for queued device work).

The entry point keeps its NTT(b) scratch in a static device array instead of
asking the context's pool for it.  This test calls it through the C ABI twice
in a row, on a fresh context whose budget is frozen at the bytes already in
use (so any pool allocation would fail), and checks each result bit for bit
against the allocating entry point vkhel_vector_polymul and against the CPU
oracle's polymul, for a 60-bit prime and for the largest NTT primes below
2^62 and below 2^63 (the top of each of the two kernel families' ranges).
The tolerance is zero: the products are integer arithmetic.  The file is
named to be collected last and uses only its own context, so it passes alone
or after the rest of the suite.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("qbound", [1 << 60, 1 << 62, 1 << 63])
@pytest.mark.parametrize("log_n", [8, 12, 14])
def test_noalloc_polymul_equals_allocating_polymul(vk, oracle, log_n, qbound):
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1, bound=qbound)[0]
    w = workloads.root_for(n, q)
    rng = np.random.default_rng(1000 + log_n)
    with vk.Context() as ctx:
        t = vk.NttTables(n, q, w)
        a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
        a, b = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h)
        ref, got = vk.Vector(ctx, n), vk.Vector(ctx, n)
        vk.polymul(a, b, ref, t)  # allocating entry point; also makes the tables resident
        ctx.set_budget(ctx.bytes_in_use)  # from here on no pool allocation can succeed
        in_use = ctx.bytes_in_use
        for call in range(2):  # two calls in a row share the static scratch
            if call == 1:
                a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
                a.upload(a_h)
                b.upload(b_h)
                vk.polymul(a, b, ref, t)
            vk.polymul_noalloc(a, b, got, t)
            g = got.download()
            np.testing.assert_array_equal(g, ref.download(), err_msg=f"call {call}")
            want, st = oracle.polymul(a_h, b_h, n, q, w)
            assert st == 0
            np.testing.assert_array_equal(g, want, err_msg=f"call {call} vs the oracle")
        # result aliasing an operand is fine: the scratch is separate
        vk.polymul_noalloc(a, b, a, t)
        np.testing.assert_array_equal(a.download(), ref.download())
        assert ctx.bytes_in_use == in_use


def test_noalloc_polymul_rejects_what_it_cannot_do(vk):
    with vk.Context() as ctx:
        n = 1 << 15  # beyond the static scratch
        q = workloads.ntt_primes(n, 1)[0]
        t = vk.NttTables(n, q, workloads.root_for(n, q))
        v = vk.Vector(ctx, n)
        with pytest.raises(vk.VkhelError) as e:
            vk.polymul_noalloc(v, v, v, t)
        assert e.value.code == 8 and "static scratch" in e.value.msg
        n = 1 << 12  # tables never uploaded on this context
        q = workloads.ntt_primes(n, 1)[0]
        t = vk.NttTables(n, q, workloads.root_for(n, q))
        v = vk.Vector(ctx, n)
        with pytest.raises(vk.VkhelError) as e:
            vk.polymul_noalloc(v, v, v, t)
        assert e.value.code == 1 and "not resident" in e.value.msg
