"""Bit-exact parity of every GPU operation with the CPU oracle.

Seeded random inputs at sizes the oracle finishes in seconds, edge values,
unreduced inputs, in-place and out-of-place calls, vectors longer than n, and
size-independent properties (round trips, schoolbook products) at the largest
supported degrees.  The bar is bit-exact equality: every operation here is
integer arithmetic.
"""
import numpy as np
import pytest

from conftest import u64
from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1

# moduli covering 2-bit .. 64-bit, primes and composites (element-wise ops
# accept any modulus >= 2)
ELEM_MODS = [2, 3, 5, 10, 769, 65537, (1 << 20) + 7, 1125891450734593, 2251799813685313,
             1152921504606748673, 2305843009211596801, (1 << 62) - 57, (1 << 63) + 29, M64]

LENGTHS = [1, 2, 3, 17, 1000, 4097, (1 << 20) + 3]


def rand64(rng, n):
    return rng.integers(0, M64, size=n, dtype=np.uint64, endpoint=True)


def edge_values(q):
    vals = [0, 1, 2, q - 2, q - 1, q, q + 1, 2 * q - 1, 2 * q, 4 * q - 1, M64, M64 - 1, 1 << 63, (1 << 62) - 1]
    return u64([v & M64 for v in vals if v >= 0])


def operands(rng, q, n):
    a, b = rand64(rng, n), rand64(rng, n)
    e = edge_values(q)
    k = min(len(e), n)
    a[:k] = e[:k]
    b[:k] = e[::-1][:k]
    return a, b


@pytest.mark.parametrize("mod", ELEM_MODS)
@pytest.mark.parametrize("n", [3, 4097])
def test_elementwise_ops_match_oracle(vk, ctx, oracle, mod, n):
    rng = np.random.default_rng(mod % 100003 + n)
    a_h, b_h = operands(rng, mod, n)
    a, b, r = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    m = int(rng.integers(0, M64, dtype=np.uint64, endpoint=True))
    for mult in (1, 2, mod - 1, m % mod, m):
        vk.elemfma(a, b, r, mult, mod)
        np.testing.assert_array_equal(r.download(), oracle.elemfma(a_h, b_h, mult, mod), err_msg=f"fma m={mult}")
        vk.elemfma_canonical(a, b, r, mult, mod)
        np.testing.assert_array_equal(r.download(), oracle.elemfma_canonical(a_h, b_h, mult, mod))
    vk.elemmul(a, b, r, mod)
    np.testing.assert_array_equal(r.download(), oracle.elemmul(a_h, b_h, mod))
    for bound, diff in ((mod // 2, mod), (0, 1), (M64, 5), (int(a_h[-1]), M64)):
        vk.elemgtsub(a, r, bound, diff, mod)
        np.testing.assert_array_equal(r.download(), oracle.elemgtsub(a_h, bound, diff, mod))
        vk.elemgtadd(a, r, bound, diff)
        np.testing.assert_array_equal(r.download(), oracle.elemgtadd(a_h, bound, diff))
    for q in (M64, mod, 73):
        vk.elemmod(a, r, mod, q)
        np.testing.assert_array_equal(r.download(), oracle.elemmod(a_h, mod, q))


@pytest.mark.parametrize("length", LENGTHS)
def test_elementwise_lengths_and_in_place(vk, ctx, oracle, length):
    q = 1152921504606748673
    rng = np.random.default_rng(length)
    a_h, b_h = rand64(rng, length), rand64(rng, length)
    a, b = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h)
    vk.elemmul(a, b, a, q)  # in place, result aliases an operand
    np.testing.assert_array_equal(a.download(), oracle.elemmul(a_h, b_h, q))
    c = vk.Vector(ctx, b_h)
    vk.elemfma(c, c, c, 12345, q)
    np.testing.assert_array_equal(c.download(), oracle.elemfma(b_h, b_h, 12345, q))


def test_elementwise_result_shorter_than_operands(vk, ctx, oracle):
    # length comes from `result` (src/kernels/elemmul.c:164)
    q = 769
    rng = np.random.default_rng(1)
    a_h, b_h = rand64(rng, 100), rand64(rng, 100)
    a, b, r = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, 37)
    vk.elemmul(a, b, r, q)
    np.testing.assert_array_equal(r.download(), oracle.elemmul(a_h[:37], b_h[:37], q))


def test_elementwise_rejects_bad_arguments(vk, ctx):
    a, r = vk.Vector(ctx, 10), vk.Vector(ctx, 20)
    with pytest.raises(vk.VkhelError):
        vk.elemmul(a, a, r, 17)  # operand shorter than result
    with pytest.raises(vk.VkhelError):
        vk.elemmul(r, r, a, 1)  # modulus < 2
    with pytest.raises(vk.VkhelError):
        vk.elemgtsub(r, a, 1, 1, 0)


TRANSFORM_BITS = [17, 31, 50, 60, 61, 62]


def ntt_params(n, bits):
    q = workloads.ntt_primes(n, 1, bound=1 << bits)[0]
    return q, workloads.root_for(n, q)


@pytest.mark.parametrize("log_n", list(range(1, 21)))
@pytest.mark.parametrize("bits", [31, 60, 62, 63])
def test_transforms_match_oracle(vk, ctx, oracle, log_n, bits):
    """Every degree 2..2^20 (one CTA, a cluster, passes over HBM) for 31- to
    63-bit primes; the 63-bit ones (2^62 <= q < 2^63) run the [0, 2q) kernel
    family, and below 2^63 by a little the reference's own table products
    overflow, so its tables are not the powers of w (they are reproduced)."""
    n = 1 << log_n
    if bits == 31 and n >= 1 << 14:
        bits = 40
    q, w = ntt_params(n, bits)
    t = vk.NttTables(n, q, w)
    ot = oracle.tables(n, q, w)
    rng = np.random.default_rng(log_n * 100 + bits)
    a_h = workloads.uniform(rng, q, n)
    a, r = vk.Vector(ctx, a_h), vk.Vector(ctx, n)
    vk.forward_transform(a, r, t)
    f_ref, st = oracle.forward(a_h, n, q, w, ot)
    assert st == 0
    np.testing.assert_array_equal(r.download(), f_ref)
    vk.inverse_transform(r, a, t)
    np.testing.assert_array_equal(a.download(), a_h)
    # in place
    v = vk.Vector(ctx, f_ref)
    vk.inverse_transform(v, v, t)
    np.testing.assert_array_equal(v.download(), a_h)
    vk.forward_transform(v, v, t)
    np.testing.assert_array_equal(v.download(), f_ref)


@pytest.mark.parametrize("bits", [61, 63])
@pytest.mark.parametrize("log_n", [1, 3, 7, 8, 10, 13, 14, 15, 16, 18, 19])
def test_forward_unreduced_inputs_match_oracle(vk, ctx, oracle, log_n, bits):
    # the first reference stage wraps (X + WY) at 2^64 before reducing
    n = 1 << log_n
    q, w = ntt_params(n, bits)
    rng = np.random.default_rng(log_n)
    a_h = rand64(rng, n)
    a_h[: min(n, 8)] = edge_values(q)[: min(n, 8)]
    t = vk.NttTables(n, q, w)
    a, r = vk.Vector(ctx, a_h), vk.Vector(ctx, n)
    vk.forward_transform(a, r, t)
    f_ref, st = oracle.forward(a_h, n, q, w)
    assert st == 0
    np.testing.assert_array_equal(r.download(), f_ref)


@pytest.mark.parametrize("bits", [60, 63])
@pytest.mark.parametrize("log_n", [1, 4, 8, 11, 14, 15, 18, 19])
def test_inverse_unreduced_inputs_match_oracle(vk, ctx, oracle, log_n, bits):
    # inputs below 2^62 (the reference's subtraction loop terminates) plus
    # pairs whose sum wraps 2^64 with a small second element
    n = 1 << log_n
    q, w = ntt_params(n, bits)
    rng = np.random.default_rng(log_n + 7)
    a_h = rng.integers(0, 1 << 62, size=n, dtype=np.uint64)
    if n >= 4:
        a_h[0], a_h[1] = M64 - 3, 5
        a_h[2], a_h[3] = (1 << 63) + 11, 1 << 10
    t = vk.NttTables(n, q, w)
    a, r = vk.Vector(ctx, a_h), vk.Vector(ctx, n)
    vk.inverse_transform(a, r, t)
    i_ref, st = oracle.inverse(a_h, n, q, w)
    assert st == 0
    np.testing.assert_array_equal(r.download(), i_ref)


def test_transform_vectors_longer_than_n(vk, ctx, oracle):
    # forward leaves words past n alone; inverse scales all result->length
    # words by n^-1 (src/vector.c:635-638)
    n = 1024
    q, w = ntt_params(n, 60)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(3)
    a_h = workloads.uniform(rng, q, n + 100)
    r0 = rand64(rng, n + 100)
    a, r = vk.Vector(ctx, a_h), vk.Vector(ctx, r0)
    vk.forward_transform(a, r, t)
    got = r.download()
    np.testing.assert_array_equal(got[:n], oracle.forward(a_h, n, q, w)[0])
    np.testing.assert_array_equal(got[n:], r0[n:])
    r = vk.Vector(ctx, r0)
    vk.inverse_transform(a, r, t)
    got = r.download()
    np.testing.assert_array_equal(got[:n], oracle.inverse(a_h, n, q, w)[0])
    np.testing.assert_array_equal(got[n:], oracle.elemmulconst(r0[n:], oracle.invmod(n, q), q))


def test_transform_degree_one(vk, ctx, oracle):
    # n = 1: the stage loops run zero times; inverse still scales result
    q, w = 97, 96
    t = vk.NttTables(1, q, w)
    a, r = vk.Vector(ctx, u64([5])), vk.Vector(ctx, u64([1000]))
    vk.forward_transform(a, r, t)
    assert int(r.download()[0]) == 1000
    vk.inverse_transform(a, r, t)
    assert int(r.download()[0]) == 1000 % 97


def test_transform_rejects_unsupported(vk, ctx):
    n = 16
    t = vk.NttTables(n, (1 << 63) + 1, 3)  # the reference's inverse-mod needs q < 2^63
    a = vk.Vector(ctx, 64)
    with pytest.raises(vk.VkhelError) as e:
        vk.forward_transform(a, a, t)
    assert e.value.code == 8
    # a 63-bit modulus whose reference table builder leaves an entry >= q
    # (its Barrett product overflows): refused rather than computed lazily
    t = vk.NttTables(64, 8735340036816624049, 8488042347404613068)
    assert (t.arrays()["roots"] >= t.q).any()
    with pytest.raises(vk.VkhelError) as e:
        vk.forward_transform(a, a, t)
    assert e.value.code == 8 and "not below q" in e.value.msg
    t = vk.NttTables(128, 2251799813685313, 3)
    with pytest.raises(vk.VkhelError):
        vk.forward_transform(a, a, t)  # vector shorter than n


@pytest.mark.parametrize("log_n", [17, 22, 24, 26])
def test_round_trip_largest_degree(vk, ctx, log_n):
    n = 1 << log_n
    # 62- and 63-bit tables are built on the host (63-bit: one extended-Euclid
    # inverse per entry, as the reference does), seconds at 2^24
    for bits in (40, 60, 62, 63) if log_n < 24 else (40, 60) if log_n < 26 else (60,):
        q, w = ntt_params(n, bits)
        t = vk.NttTables(n, q, w)
        a_h = workloads.uniform(np.random.default_rng(bits), q, n)
        v = vk.Vector(ctx, a_h)
        vk.forward_transform(v, v, t)
        assert (v.download() < q).all()
        vk.inverse_transform(v, v, t)
        np.testing.assert_array_equal(v.download(), a_h)


@pytest.mark.parametrize("log_n", [18, 22, 26])
def test_polymul_by_a_monomial_is_a_negacyclic_rotation(vk, ctx, log_n):
    """At degrees the oracle is too slow for, the product with X^k is exactly
    known: a rotated by k with the k wrapped words negated mod q (X^n = -1).
    Checked through the composed path (n >= 2^18) up to the largest degree."""
    n = 1 << log_n
    q, w = ntt_params(n, 60)
    rng = np.random.default_rng(log_n)
    t = vk.NttTables(n, q, w)
    a_h = workloads.uniform(rng, q, n)
    for k in (1, int(rng.integers(2, n))):
        b_h = np.zeros(n, np.uint64)
        b_h[k] = 1
        a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
        vk.polymul(a, b, c, t)
        want = np.empty(n, np.uint64)
        want[k:] = a_h[:n - k]
        tail = a_h[n - k:]
        want[:k] = np.where(tail == 0, np.uint64(0), np.uint64(q) - tail)
        np.testing.assert_array_equal(c.download(), want, err_msg=f"X^{k}")


@pytest.mark.parametrize("bits", [60, 63])
@pytest.mark.parametrize("log_n", [1, 2, 4, 7, 8, 9, 10, 12, 13, 14, 15, 16, 17, 18, 20])
def test_polymul_matches_reference_composition(vk, ctx, oracle, log_n, bits):
    """The fused (2^8..2^17) and composed (other n) products equal the
    reference's forward, forward, elemmul, inverse; at 63 bits elemmul's
    Barrett estimate overflows for large products and the kernels reproduce
    its words."""
    n = 1 << log_n
    q, w = ntt_params(n, bits)
    t = vk.NttTables(n, q, w)
    rng = np.random.default_rng(log_n + 40)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    a_h[0] = M64  # an unreduced coefficient takes the exact first-stage path
    ref, st = oracle.polymul(a_h, b_h, n, q, w)
    assert st == 0
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    vk.polymul(a, b, c, t)
    np.testing.assert_array_equal(c.download(), ref)
    vk.polymul(a, b, a, t)  # result aliases a
    np.testing.assert_array_equal(a.download(), ref)
    a = vk.Vector(ctx, a_h)
    vk.polymul(a, b, b, t)  # result aliases b
    np.testing.assert_array_equal(b.download(), ref)


@pytest.mark.parametrize("log_n", [3, 8, 9])
def test_polymul_is_negacyclic_schoolbook(vk, ctx, oracle, log_n):
    n = 1 << log_n
    q, w = ntt_params(n, 61)
    rng = np.random.default_rng(log_n)
    a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
    a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
    vk.polymul(a, b, c, vk.NttTables(n, q, w))
    np.testing.assert_array_equal(c.download(), oracle.schoolbook(a_h, b_h, n, q))


def test_zero_length_results(vk, ctx):
    """Zero-length vectors, which the reference allows: every element-wise op
    with a zero-length result does nothing and reports no error, also with
    longer operands; the vectors download as empty arrays."""
    q = (1 << 61) - 1
    a, b, r = vk.Vector(ctx, 0), vk.Vector(ctx, 0), vk.Vector(ctx, 0)
    x = vk.Vector(ctx, np.arange(1, 9, dtype=np.uint64))
    for p, s in ((a, b), (x, x)):
        vk.elemmul(p, s, r, q)
        vk.elemfma(p, s, r, 3, q)
        vk.elemfma_canonical(p, s, r, 3, q)
        vk.elemgtadd(p, r, 1, 2)
        vk.elemgtsub(p, r, 1, 2, q)
        vk.elemmod(p, r, 65537, q)
        vk.elemmod(p, r, 2, q)
    assert r.download().size == 0 and a.download().size == 0
    np.testing.assert_array_equal(x.download(), np.arange(1, 9, dtype=np.uint64))
