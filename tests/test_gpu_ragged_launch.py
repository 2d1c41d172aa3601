"""A ragged batch as one persistent launch (k_polymul_ragged).

With tuning entry (family 3, log_n 2) = 1, a committed batch whose classes
are all fused limb products of degrees 2^12 .. 2^16 (q < 2^62, no epilogue)
runs as a single kernel: clusters of four CTAs take the 2^16 products and
pairs of 2^15 products, then each CTA takes 2^14, 2^13 and pairs of 2^12
products.  Every limb product must equal the oracle's and the per-class
launches' words; odd counts of 2^15 and 2^12 products exercise the dummy
copy that completes a pair.  Batches the single launch does not cover (an
epilogue, a 63-bit modulus, another degree) keep the per-class kernels.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture
def single_launch(vk):
    L = vk.lib()
    saved = L.vkhel_tune_get(3, 2)
    L.vkhel_tune_set(3, 2, 1)
    yield
    L.vkhel_tune_set(3, 2, saved)


def _instances(vk, shapes, seed):
    rng = np.random.default_rng(seed)
    tabs, out = {}, []
    for log_n, limbs in shapes:
        n = 1 << log_n
        qs = workloads.ntt_primes(n, limbs)
        ws = [workloads.root_for(n, q) for q in qs]
        for q, w in zip(qs, ws):
            tabs.setdefault((n, q), vk.NttTables(n, q, w))
        a = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        b = np.concatenate([workloads.uniform(rng, q, n) for q in qs])
        out.append((n, qs, ws, a, b, [tabs[(n, q)] for q in qs]))
    return out, tabs


def _run(vk, ctx, inst, graph, lift=None):
    outs = [vk.Vector(ctx, len(qs) * n) for n, qs, ws, a, b, t in inst]
    ins = [(vk.Vector(ctx, a), vk.Vector(ctx, b)) for n, qs, ws, a, b, t in inst]
    bt = vk.Batch(ctx)
    for (n, qs, ws, a, b, t), (va, vb), vc in zip(inst, ins, outs):
        bt.add_polymul(t, va, vb, vc, lift=lift)
    bt.commit(graph=graph)
    bt.run()
    kernels = bt.kernels
    bt.close()
    return [v.download() for v in outs], kernels


def _check(oracle, inst, got):
    for i, (n, qs, ws, a, b, _) in enumerate(inst):
        ref, _ = oracle.polymul_batch(a.reshape(-1, n), b.reshape(-1, n), n, qs, ws,
                                      np.arange(len(qs), dtype=np.uint32))
        np.testing.assert_array_equal(got[i].reshape(-1, n), ref, err_msg=f"instance {i} (n={n})")


# odd numbers of 2^15 and of 2^12 limb products (7 and 5), even ones too
SHAPES = [(16, 2), (15, 3), (14, 2), (13, 1), (12, 3), (15, 4), (16, 1), (12, 2), (13, 3), (14, 1)]


@pytest.mark.parametrize("graph", [True, False])
def test_single_launch_matches_oracle_and_per_class(vk, ctx, oracle, single_launch, graph):
    inst, _ = _instances(vk, SHAPES, seed=5)
    got, kernels = _run(vk, ctx, inst, graph)
    assert kernels == 1
    _check(oracle, inst, got)
    vk.lib().vkhel_tune_set(3, 2, 0)
    ref, kernels_per_class = _run(vk, ctx, inst, graph)
    assert kernels_per_class == 5
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


def test_single_launch_replays_with_new_operands(vk, ctx, oracle, single_launch):
    inst, _ = _instances(vk, [(16, 1), (15, 1), (12, 1), (14, 2)], seed=6)
    outs = [vk.Vector(ctx, len(qs) * n) for n, qs, ws, a, b, t in inst]
    ins = [(vk.Vector(ctx, a), vk.Vector(ctx, b)) for n, qs, ws, a, b, t in inst]
    bt = vk.Batch(ctx)
    for (n, qs, ws, a, b, t), (va, vb), vc in zip(inst, ins, outs):
        bt.add_polymul(t, va, vb, vc)
    bt.commit(graph=True)
    assert bt.kernels == 1
    for rep in range(3):
        if rep:
            inst2, _ = _instances(vk, [(16, 1), (15, 1), (12, 1), (14, 2)], seed=60 + rep)
            inst = [(n, qs, ws, a2, b2, t) for (n, qs, ws, _, _, t), (_, _, _, a2, b2, _) in zip(inst, inst2)]
            for (n, qs, ws, a, b, t), (va, vb) in zip(inst, ins):
                va.upload(a)
                vb.upload(b)
        bt.run()
        _check(oracle, inst, [v.download() for v in outs])
    bt.close()


def test_config4_batch_as_one_launch(vk, ctx, oracle, single_launch):
    """The ragged workload itself (512 instances, seed 3): 4225 limb products."""
    inst = workloads.ragged_batch(512, seed=3)
    tabs = {}
    full = []
    for n, qs, ws, a, b in inst:
        for q, w in zip(qs, ws):
            tabs.setdefault((n, q), vk.NttTables(n, q, w))
        full.append((n, qs, ws, a, b, [tabs[(n, q)] for q in qs]))
    got, kernels = _run(vk, ctx, full, True)
    assert kernels == 1
    by_n = {}
    for i, (n, qs, ws, a, b, _) in enumerate(full):
        by_n.setdefault(n, []).append(i)
    for n, idx in by_n.items():
        top = max(idx, key=lambda i: len(full[i][1]))
        qs, ws = full[top][1], full[top][2]
        ref, _ = oracle.polymul_batch(np.concatenate([full[i][3].reshape(-1, n) for i in idx]),
                                      np.concatenate([full[i][4].reshape(-1, n) for i in idx]), n, qs, ws,
                                      np.concatenate([np.arange(len(full[i][1]), dtype=np.uint32) for i in idx]),
                                      tables=oracle.batch_tables(n, qs, ws))
        np.testing.assert_array_equal(np.concatenate([got[i].reshape(-1, n) for i in idx]), ref,
                                      err_msg=f"degree {n}")


def test_batches_outside_the_single_launch_keep_per_class_kernels(vk, ctx, oracle, single_launch):
    inst, _ = _instances(vk, [(16, 1), (12, 2)], seed=7)
    got, kernels = _run(vk, ctx, inst, True, lift=[("elemmod", 65537, 0)])  # an epilogue
    assert kernels == 2
    inst, _ = _instances(vk, [(17, 1), (12, 2)], seed=8)  # a degree above 2^16
    got, kernels = _run(vk, ctx, inst, True)
    assert kernels == 2
    _check(oracle, inst, got)
