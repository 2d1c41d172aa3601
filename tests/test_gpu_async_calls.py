"""Stream-ordered single calls (vkhel_ctx_set_async).

With the switch on, the reference's call pattern -- forward, forward,
elemmul, inverse, then the centred-lift element-wise ops, one call each --
returns before the GPU finishes, and the calls run back to back on the
context stream.  The words must be the oracle's, read back through the
reference's own map (which waits), through download, and after host copies
that overwrite an operand between queued calls; argument errors are still
reported by the call that makes them.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("log_n", [4, 12, 14, 16, 18])
def test_queued_reference_call_pattern_matches_oracle(vk, oracle, log_n):
    n = 1 << log_n
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    rng = np.random.default_rng(60 + log_n)
    with vk.Context() as ctx:
        ctx.set_async(True)
        t = vk.NttTables(n, q, w)
        a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
        a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
        rounds = []
        for r in range(3):
            vk.forward_transform(a, a, t)
            vk.forward_transform(b, b, t)
            vk.elemmul(a, b, c, q)
            vk.inverse_transform(c, c, t)
            vk.elemmod(c, c, 65537, q)
            vk.elemgtadd(c, c, 3, 1 << 20)
            got = c.map_read()  # the reference's map: waits for the queued calls
            want = oracle.polymul(a_h, b_h, n, q, w)[0]
            want = oracle.elemgtadd(oracle.elemmod(want, 65537, q), 3, 1 << 20)
            np.testing.assert_array_equal(got, want, err_msg=f"round {r}")
            # new operands through the host while nothing is queued, then again
            a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
            a.upload(a_h)
            b.upload(b_h)
            rounds.append(r)
        # a host copy between queued calls lands after the calls before it
        vk.forward_transform(a, c, t)
        a.upload(b_h)                     # overwrites a after the queued forward read it
        vk.forward_transform(a, b, t)
        np.testing.assert_array_equal(c.download(), oracle.forward(a_h, n, q, w)[0])
        np.testing.assert_array_equal(b.download(), oracle.forward(b_h, n, q, w)[0])
        with pytest.raises(vk.VkhelError):  # argument checks stay synchronous
            vk.polymul(a, b, vk.Vector(ctx, n // 2), t)
        ctx.set_async(False)


def test_many_queued_calls_then_sync(vk, oracle):
    """200 queued in-place transforms, then one wait: forward and inverse
    alternate, so the vector ends where it started."""
    n = 1 << 13
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    x_h = workloads.uniform(np.random.default_rng(7), q, n)
    with vk.Context() as ctx:
        ctx.set_async(True)
        t = vk.NttTables(n, q, w)
        x = vk.Vector(ctx, x_h)
        before = vk.launch_count()
        for _ in range(100):
            vk.forward_transform(x, x, t)
            vk.inverse_transform(x, x, t)
        assert vk.launch_count() - before >= 200
        ctx.sync()
        np.testing.assert_array_equal(x.download(), x_h)
