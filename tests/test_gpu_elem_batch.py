"""Element-wise batch: ragged independent jobs in one launch.

Each job must give exactly what the oracle's restatement of the matching
reference op gives on the same words, whatever the job's length (empty, odd,
one chunk +- 1, several chunks), pointer alignment (16-byte vector path or
8-byte scalar path), or placement (in place or not); commit must reject a
batch in which one job writes memory that another reads or writes.
"""
import numpy as np
import pytest

from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

Q = (1 << 61) - 1            # prime modulus
Q50 = workloads.ntt_primes(1024, 1, bound=1 << 50)[0]
M64 = (1 << 64) - 59         # 64-bit modulus: the exact-remainder path of fma_canonical


def _cases():
    # (op, params, binary, length, operand range)
    return [
        ("elemfma", (12345678901, Q), True, 4097, Q),
        ("elemfma", (3, Q50), True, 1, 1 << 64),                  # the shader's wrap on full-range words
        ("elemfma_canonical", (M64 - 3, M64), True, 4096, 1 << 64),
        ("elemfma_canonical", ((1 << 64) - 1, Q50), True, 10000, 1 << 64),
        ("elemmul", (Q,), True, 4095, 1 << 64),
        ("elemmul", (Q50,), True, 3, Q50),
        ("elemmulconst", (987654321, Q50), False, 65537, Q50),
        ("elemmod", (65537, Q), False, 9000, Q),
        ("elemmod", (2, Q50), False, 2, Q50),
        ("elemgtadd", (Q // 2, (1 << 64) - 17), False, 5000, Q),
        ("elemgtsub", (Q // 3, Q + 5, 1 << 40), False, (1 << 20) + 3, 1 << 64),
        ("elemgtsub", (0, 0, 2), False, 0, Q),                     # empty job
    ]


def _oracle(oracle, op, a, b, params):
    if op == "elemfma":
        return oracle.elemfma(a, b, *params)
    if op == "elemfma_canonical":
        return oracle.elemfma_canonical(a, b, *params)
    if op == "elemmul":
        return oracle.elemmul(a, b, *params)
    if op == "elemmulconst":
        return oracle.elemmulconst(a, *params)
    if op == "elemmod":
        return oracle.elemmod(a, *params)
    if op == "elemgtadd":
        return oracle.elemgtadd(a, *params)
    return oracle.elemgtsub(a, *params)


def _rand(rng, hi, n):
    if hi >= 1 << 64:
        return rng.integers(0, 1 << 64, size=n, dtype=np.uint64, endpoint=False)
    return workloads.uniform(rng, hi, n)


@pytest.mark.parametrize("graph", [True, False])
def test_ragged_batch_matches_oracle(vk, ctx, oracle, graph):
    rng = np.random.default_rng(11 + graph)
    eb = vk.ElemBatch(ctx)
    checks = []
    for i, (op, params, binary, n, hi) in enumerate(_cases()):
        a_h, b_h = _rand(rng, hi, n), _rand(rng, hi, n)
        ref = _oracle(oracle, op, a_h, b_h, params) if n else np.zeros(0, np.uint64)
        mode = i % 3
        if mode == 0:            # vectors, separate result
            a, b, r = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
            eb.add(op, a, b if binary else None, r, *params)
            checks.append((lambda r=r: r.download(), ref, op, (a, b)))
        elif mode == 1:          # in place on a
            a, b = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h)
            eb.add(op, a, b if binary else None, a, *params)
            checks.append((lambda a=a: a.download(), ref, op, (b,)))
        else:                    # raw pointers one word into each buffer: 8-byte aligned only
            seven = np.array([7], np.uint64)
            a = vk.Vector(ctx, np.concatenate([seven, a_h]))
            b = vk.Vector(ctx, np.concatenate([seven, b_h]))
            r = vk.Vector(ctx, np.full(n + 2, 99, np.uint64))
            eb.add(op, a.device_ptr + 8, b.device_ptr + 8 if binary else None, (r.device_ptr + 8, n), *params)
            checks.append((lambda r=r, n=n: r.download()[1:n + 1], ref, op, (a, b, r)))
            checks.append((lambda r=r, n=n: r.download()[[0, n + 1]], np.array([99, 99], np.uint64), "guard", ()))
    assert eb.jobs == len(_cases())
    eb.commit(graph=graph)
    eb.run()
    for get, ref, op, _ in checks:
        np.testing.assert_array_equal(get(), ref, err_msg=op)
    eb.close()


def test_batch_replays_read_fresh_operands(vk, ctx, oracle):
    rng = np.random.default_rng(3)
    n = 20000
    a_h, b_h = _rand(rng, Q, n), _rand(rng, Q, n)
    a, b, r = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    eb = vk.ElemBatch(ctx)
    eb.add("elemmul", a, b, r, Q)
    eb.commit(graph=True)
    for _ in range(3):
        a_h = _rand(rng, Q, n)
        a.upload(a_h)
        eb.run()
        np.testing.assert_array_equal(r.download(), oracle.elemmul(a_h, b_h, Q))


def test_commit_rejects_dependent_jobs(vk, ctx):
    n = 1000
    x, y, z, u = vk.Vector(ctx, 2 * n), vk.Vector(ctx, n), vk.Vector(ctx, n), vk.Vector(ctx, n)
    # writes overlap
    eb = vk.ElemBatch(ctx)
    eb.add("elemgtadd", y, None, (x.device_ptr, n), 1, 1)
    eb.add("elemgtadd", z, None, (x.device_ptr + 8 * (n - 1), n), 1, 1)
    with pytest.raises(vk.VkhelError):
        eb.commit()
    # one job reads what another writes
    eb = vk.ElemBatch(ctx)
    eb.add("elemmod", y, None, z, 3, Q)
    eb.add("elemmul", z, y, u, Q)
    with pytest.raises(vk.VkhelError):
        eb.commit()
    # in place and disjoint halves are fine
    eb = vk.ElemBatch(ctx)
    eb.add("elemmod", y, None, y, 3, Q)
    eb.add("elemgtadd", z, None, (x.device_ptr, n), 1, 1)
    eb.add("elemgtadd", z, None, (x.device_ptr + 8 * n, n), 1, 1)
    eb.commit()
    eb.run()


def test_add_rejects_bad_jobs(vk, ctx):
    a, r = vk.Vector(ctx, 8), vk.Vector(ctx, 8)
    eb = vk.ElemBatch(ctx)
    for op, params in (("elemmul", (1,)), ("elemgtsub", (1, 1, 0)), (99, (1, 1, 1)), ("elemfma", (1, 0))):
        with pytest.raises(vk.VkhelError):
            eb.add(op, a, a, r, *params)
    with pytest.raises(vk.VkhelError):
        eb.add("elemmul", a, None, r, 17)       # binary op without b
    with pytest.raises(vk.VkhelError):
        eb.commit()                             # nothing was added
