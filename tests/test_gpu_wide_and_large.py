"""The top of the modulus range and the degrees past one cluster, through the
batch, lift and server paths.

Moduli 2^62 <= q < 2^63 run their own kernel family ([0, 2q) butterflies);
a batch or a server micro-batch whose limbs mix them with smaller moduli is
split into one class per (degree, modulus class).  Degrees n >= 2^18 run
passes over HBM around 2^14-word sub-blocks.  Everything is compared with
the oracle's restatement of the reference (forward, forward, elemmul,
inverse per limb product; the element-wise ops after it for a lift), bit for
bit.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


def _prime(n, bits, k=0):
    return workloads.ntt_primes(n, k + 1, bound=1 << bits)[k]


def _mixed_primes(n):
    """Four limbs: 60-, 63-, 62- and 63-bit primes (two classes)."""
    return [_prime(n, 60), _prime(n, 63), _prime(n, 62), _prime(n, 63, 1)]


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("log_n", [6, 10, 14, 16, 17, 19])
def test_batch_mixes_modulus_classes(vk, ctx, oracle, log_n, graph):
    n = 1 << log_n
    qs = _mixed_primes(n)
    ws = [workloads.root_for(n, q) for q in qs]
    tabs = [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]
    rng = np.random.default_rng(log_n)
    a_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
    b_h = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, 4 * n)
    fa, ia = vk.Vector(ctx, 4 * n), vk.Vector(ctx, 4 * n)
    bt = vk.Batch(ctx)
    bt.add_polymul(tabs, a, b, c)
    bt.add_transform(tabs, a, fa)
    bt.add_transform(tabs, a, ia, inverse=True, lift=[("elemmod", 65537, 0)])
    bt.commit(graph=graph)
    bt.run()
    bt.close()
    got_c, got_f, got_i = (v.download().reshape(4, n) for v in (c, fa, ia))
    for k, (q, w) in enumerate(zip(qs, ws)):
        ref, st = oracle.polymul(a_h[k * n:(k + 1) * n], b_h[k * n:(k + 1) * n], n, q, w)
        assert st == 0
        np.testing.assert_array_equal(got_c[k], ref, err_msg=f"product limb {k} ({q.bit_length()} bits)")
        np.testing.assert_array_equal(got_f[k], oracle.forward(a_h[k * n:(k + 1) * n], n, q, w)[0])
        inv = oracle.inverse(a_h[k * n:(k + 1) * n], n, q, w)[0]
        np.testing.assert_array_equal(got_i[k], oracle.elemmod(inv, 65537, q), err_msg=f"inverse+lift limb {k}")


@pytest.mark.parametrize("log_n", [8, 12, 14, 15, 17])
def test_polymul_lift_with_63_bit_moduli(vk, ctx, oracle, log_n):
    n = 1 << log_n
    q = _prime(n, 63)
    w = workloads.root_for(n, q)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(300 + log_n)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    ref, _ = oracle.polymul(a_h, b_h, n, q, w)
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    steps = [("elemmod", 65537, 0), ("elemgtadd", 32768, 3)]
    vk.polymul_lift(a, b, c, t, steps)
    want = oracle.elemgtadd(oracle.elemmod(ref, 65537, q), 32768, 3)
    np.testing.assert_array_equal(c.download(), want)


def test_server_mixes_modulus_classes_and_large_degrees(vk, oracle):
    """Requests with 63-bit limbs beside 60-bit ones and degrees 2^12 .. 2^19
    in one server; each result against the oracle, alone and in the mix."""
    rng = np.random.default_rng(44)
    reqs = []
    for log_n in (12, 14, 16, 17, 18, 19):
        n = 1 << log_n
        qs = _mixed_primes(n)[: 2 + log_n % 3]
        ws = [workloads.root_for(n, q) for q in qs]
        a = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        b = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        reqs.append((n, qs, ws, a, b, [vk.NttTables(n, q, w) for q, w in zip(qs, ws)]))
    mix = [np.zeros(len(r[1]) * r[0], np.uint64) for r in reqs]
    alone = [np.zeros_like(m) for m in mix]
    with vk.Server(device_budget=8 << 30) as srv:
        ids = [srv.submit(tabs, a, b, c) for (n, qs, ws, a, b, tabs), c in zip(reqs, mix)]
        assert all(srv.wait(r) == 0 for r in ids)
        for (n, qs, ws, a, b, tabs), c in zip(reqs, alone):
            assert srv.wait(srv.submit(tabs, a, b, c)) == 0
    for i, (n, qs, ws, a, b, _) in enumerate(reqs):
        for k, (q, w) in enumerate(zip(qs, ws)):
            ref, _ = oracle.polymul(a[k * n:(k + 1) * n], b[k * n:(k + 1) * n], n, q, w)
            np.testing.assert_array_equal(mix[i][k * n:(k + 1) * n], ref, err_msg=f"request {i} limb {k}")
        np.testing.assert_array_equal(alone[i], mix[i])


@pytest.mark.parametrize("log_n", [18, 21])
def test_large_degree_inverse_lift_and_in_place(vk, ctx, oracle, log_n):
    n = 1 << log_n
    q = _prime(n, 60)
    w = workloads.root_for(n, q)
    t = vk.NttTables(n, q, w)
    a_h = workloads.uniform(np.random.default_rng(log_n), q, n)
    v = vk.Vector(ctx, a_h)
    vk.forward_transform(v, v, t)
    f = oracle.forward(a_h, n, q, w)[0]
    np.testing.assert_array_equal(v.download(), f)
    vk.inverse_transform_lift(v, v, t, [("elemmod", 2, 0)])
    np.testing.assert_array_equal(v.download(), oracle.elemmod(a_h, 2, q))
