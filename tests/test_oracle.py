"""The CPU oracle against the reference's own golden vectors and known answers.

The oracle (oracle/oracle.c) is what every GPU parity test compares with, so it
is pinned here first: every operation recorded from the reference's
test/vector.c, every known answer of test/numbers.c and test/ntt.c, and the
reference's own twiddle tables (tests/golden/*.json, made by
tests/golden/make_golden.py).  Where the reference's numbers.c/ntt_tables.c
have been compiled from source in this checkout (oracle/_ref), the oracle is
also compared with them directly on random inputs.
"""
import ctypes
import hashlib
import os

import numpy as np
import pytest

from conftest import ROOT, load_golden, u64
from vkhel_gb300 import workloads

VEC = load_golden("reference_vectors.json")
NUM = load_golden("reference_numbers.json")
TAB = load_golden("reference_tables.json")


def _ints(xs):
    return u64([int(x) for x in xs])


def _replay(oracle, op):
    p = {k: int(v) for k, v in op["params"].items()}
    a = _ints(op["a"]) if "a" in op else None
    b = _ints(op["b"]) if "b" in op else None
    name = op["op"]
    if name in ("copy_from_host", "dup"):
        return a
    if name == "elemfma":
        return oracle.elemfma(a, b, p["multiplier"], p["mod"])
    if name == "elemmul":
        return oracle.elemmul(a, b, p["mod"])
    if name == "elemmod":
        return oracle.elemmod(a, p["mod"], p["q"])
    if name == "elemgtadd":
        return oracle.elemgtadd(a, p["bound"], p["diff"])
    if name == "elemgtsub":
        return oracle.elemgtsub(a, p["bound"], p["diff"], p["mod"])
    if name == "forward_transform":
        return oracle.forward(a, p["n"], p["q"], p["w"])[0]
    if name == "inverse_transform":
        return oracle.inverse(a, p["n"], p["q"], p["w"])[0]
    raise KeyError(name)


@pytest.mark.parametrize("i", range(len(VEC["ops"])))
def test_oracle_reproduces_reference_vectors(oracle, i):
    op = VEC["ops"][i]
    np.testing.assert_array_equal(_replay(oracle, op), _ints(op["expected"]))


def test_golden_vectors_cover_every_reference_test():
    ops = {o["op"] for o in VEC["ops"]}
    assert ops == {"copy_from_host", "dup", "elemfma", "elemmul", "elemmod", "elemgtadd", "elemgtsub",
                   "forward_transform", "inverse_transform"}
    for name in ("elemfma", "elemmod", "elemmul", "elemgtadd", "elemgtsub", "forward_transform_big"):
        assert name in VEC["source"]


def test_oracle_number_theory_kats(oracle):
    k = NUM["kats"]
    for a, b, m, r in k["multiply_mod"]:
        assert oracle.mulmod(int(a), int(b), int(m)) == int(r)
    for b, e, m, r in k["power_mod"]:
        assert oracle.powmod(int(b), int(e), int(m)) == int(r)
    for r, d, m, expect in k["is_primitive_root"]:
        assert oracle.is_primitive_root(int(r), int(d), int(m)) == expect
    for a, m, r in k["inverse_mod"]:
        assert oracle.invmod(int(a), int(m)) == int(r)
    for n, q, w, roots in k["ntt_roots"]:
        np.testing.assert_array_equal(oracle.tables(int(n), int(q), int(w))["roots"], _ints(roots))


def _sha(a):
    return hashlib.sha256(u64(a).astype("<u8").tobytes()).hexdigest()


@pytest.mark.parametrize("rec", TAB["tables"], ids=lambda r: f"n{r['n']}")
def test_oracle_tables_match_reference_tables(oracle, rec):
    t = oracle.tables(int(rec["n"]), int(rec["q"]), int(rec["w"]))
    for k, v in t.items():
        assert _sha(v) == rec[k + "_sha256"], k
        if k in rec:
            np.testing.assert_array_equal(v, _ints(rec[k]))


@pytest.mark.parametrize("n", [2, 4, 16, 64, 128])
def test_oracle_polymul_is_negacyclic_product(oracle, n):
    rng = np.random.default_rng(n)
    for q in workloads.ntt_primes(n, 2, bound=1 << 50) + [113 if n <= 4 else workloads.ntt_primes(n, 1, 1 << 20)[0]]:
        w = workloads.root_for(n, q)
        a, b = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
        c, st = oracle.polymul(a, b, n, q, w)
        assert st == 0
        np.testing.assert_array_equal(c, oracle.schoolbook(a, b, n, q))


def test_oracle_round_trip_and_canonical(oracle):
    n = 1024
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    a = workloads.uniform(np.random.default_rng(5), q, n)
    f, st = oracle.forward(a, n, q, w)
    assert st == 0 and (f < q).all()
    back, st = oracle.inverse(f, n, q, w)
    np.testing.assert_array_equal(back, a)


def test_oracle_elemfma_keeps_the_shader_wrap(oracle):
    # elemfma.comp:47-52 computes mod - x instead of x - mod; with a sum >= q the
    # reference output is 2^64 - (sum - q), while the canonical variant is exact.
    a, b = u64([700]), u64([100])
    ref = oracle.elemfma(a, b, 1, 769)
    can = oracle.elemfma_canonical(a, b, 1, 769)
    assert int(can[0]) == 31
    assert int(ref[0]) == (769 - 800) % (1 << 64)


REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libvkhelref.so")


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference host code not built in this checkout")
def test_oracle_matches_reference_numbers_c_on_random_inputs(oracle):
    L = ctypes.CDLL(REF_LIB)
    L.nt_multiply_mod.restype = ctypes.c_uint64
    L.nt_multiply_mod.argtypes = [ctypes.c_uint64] * 4
    L.nt_inverse_mod.restype = ctypes.c_uint64
    L.nt_inverse_mod.argtypes = [ctypes.c_uint64] * 2
    rng = np.random.default_rng(11)
    for bits in (20, 40, 50, 59, 60, 61, 62, 63):
        q = workloads.ntt_primes(1024, 1, bound=1 << bits)[0]
        for _ in range(300):
            a, b = (int(x) for x in rng.integers(0, q, 2, dtype=np.uint64))
            assert oracle.mulmod(a, b, q) == L.nt_multiply_mod(a, b, q, 0)
            if a:
                assert oracle.invmod(a, q) == L.nt_inverse_mod(a, q)


def test_reference_reduce64_returns_reduced_operands_unchanged(oracle):
    """The reference's Barrett reduce64 (elemgtsub.comp:36-47; elemgtsub with
    a bound no word exceeds returns it) gives back every x < mod unchanged,
    for moduli of every bit length; the element-wise kernels rely on this to
    skip the reduction of operands that are already reduced."""
    rng = np.random.default_rng(17)
    for bits in range(2, 65):
        lo, hi = 1 << (bits - 1), (1 << bits) - 1
        mods = {max(lo, 2), hi, lo + (hi - lo) // 2, min(hi, 3 << (bits - 2)), min(hi, (3 << (bits - 2)) + 1)}
        for mod in sorted(m for m in mods if m >= 2):
            x = rng.integers(0, mod, size=512, dtype=np.uint64)
            x[:4] = [0, mod - 1, mod // 2, (3 * mod) // 4]
            out = oracle.elemgtsub(x, (1 << 64) - 1, 0, mod)
            np.testing.assert_array_equal(out, x, err_msg=f"mod={mod}")
