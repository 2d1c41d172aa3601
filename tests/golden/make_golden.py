"""Regenerate the golden fixtures in this folder from the reference checkout.

Run from the repository root, in a container that has the reference checkout
(oracle/Makefile knows its usual location; override with VKHEL_REF=...):

    python tests/golden/make_golden.py

What it does, without copying any reference source into this repository:

1. ``make -C oracle ref`` compiles, in place, the reference's own test programs
   against the CPU oracle (test/numbers.c with oracle/nt_abi.c, test/vector.c
   with oracle/vkhel_shim.c) and the reference's numbers.c + ntt_tables.c into
   oracle/_ref/libvkhelref.so.
2. Runs test/vector.c against the oracle with VKHEL_SHIM_LOG set.  That
   program asserts every golden vector of the reference (test/vector.c:39-329);
   it exits 0 only if the oracle reproduced all of them, and the log then holds
   each operation with its inputs and the asserted outputs ->
   reference_vectors.json.
3. Reads the known-answer literals of test/numbers.c and test/ntt.c as text ->
   reference_numbers.json, and checks them against the reference's own
   numbers.c through ctypes.
4. Records the reference's own twiddle tables (ntt_tables.c) for a few
   (n, q, w) -> reference_tables.json (full arrays for small n, SHA-256 of the
   little-endian arrays for large n).
"""
import ctypes
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import pyoracle  # noqa: E402
from vkhel_gb300 import workloads  # noqa: E402

REF = pyoracle.reference_dir()
if REF is None:
    raise SystemExit("the reference checkout is not present (set VKHEL_REF=...)")


def build_ref():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"],
                   check=True)


def vector_cases():
    exe = os.path.join(ROOT, "oracle", "_ref", "test_vector_oracle")
    with tempfile.TemporaryDirectory() as td:
        log = os.path.join(td, "ops.jsonl")
        env = dict(os.environ, VKHEL_SHIM_LOG=log)
        out = subprocess.run([exe], env=env, capture_output=True, text=True)
        if out.returncode != 0:
            raise SystemExit("reference test/vector.c failed on the oracle:\n" + out.stdout + out.stderr)
        passed = [l.split()[0] for l in out.stdout.splitlines() if l.endswith("passed")]
        with open(log) as f:
            ops = [json.loads(l) for l in f]
    return passed, ops


def number_kats():
    src = open(os.path.join(REF, "test", "numbers.c")).read()
    kats = {"multiply_mod": [], "power_mod": [], "is_primitive_root": [], "inverse_mod": []}
    # test_multiply_mod: blocks that set `mod` then assert products.
    body = src[src.index("void test_multiply_mod"):src.index("void test_power_mod")]
    for block in body.split("{")[2:]:
        m = re.search(r"const uint64_t mod = (\d+);", block)
        if not m:
            continue
        mod = int(m.group(1))
        for a, b, r in re.findall(r"nt_multiply_mod\((\d+),\s*(\d+),\s*mod,\s*barrett_factor\)\s*==\s*(\d+)", block):
            kats["multiply_mod"].append([a, b, str(mod), r])
    body = src[src.index("void test_power_mod"):src.index("void test_is_primitive_root")]
    for block in body.split("{")[2:]:
        m = re.search(r"const uint64_t modulus = (0x[0-9a-fA-F]+|\d+);", block)
        if not m:
            continue
        mod = int(m.group(1), 0)
        for b, e, r in re.findall(r"nt_power_mod\((0x[0-9a-fA-F]+|\d+),\s*(0x[0-9a-fA-F]+|\d+),\s*modulus\)\s*==\s*(0x[0-9a-fA-F]+|\d+)", block):
            kats["power_mod"].append([str(int(b, 0)), str(int(e, 0)), str(mod), str(int(r, 0))])
    body = src[src.index("void test_is_primitive_root"):src.index("void test_inverse_mod")]
    mod = int(re.search(r"const uint64_t mod = (\d+);", body).group(1))
    for neg, r, d in re.findall(r"assert\((!?)nt_is_primitive_root\((\d+),\s*(\d+),\s*mod\)\)", body):
        kats["is_primitive_root"].append([r, d, str(mod), neg != "!"])
    body = src[src.index("void test_inverse_mod"):src.index("int main")]
    for a, m, r in re.findall(r"nt_inverse_mod\((\d+),\s*(\d+)\)\s*==\s*(\d+)", body):
        kats["inverse_mod"].append([a, m, r])

    ntt_src = open(os.path.join(REF, "test", "ntt.c")).read()
    n, q, w = re.search(r"vkhel_ntt_tables_create\((\d+),\s*(\d+),\s*(\d+)\)", ntt_src).groups()
    roots = re.search(r"\(uint64_t\[\]\)\s*\{([^}]*)\}", ntt_src).group(1)
    kats["ntt_roots"] = [[n, q, w, [x.strip() for x in roots.split(",") if x.strip()]]]

    # Every answer must hold for the reference's own numbers.c as well.
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvkhelref.so"))
    u64 = ctypes.c_uint64
    for f in ("nt_multiply_mod", "nt_power_mod", "nt_inverse_mod", "nt_compute_barrett_factor"):
        getattr(lib, f).restype = u64
    lib.nt_is_primitive_root.restype = ctypes.c_bool
    for a, b, m, r in kats["multiply_mod"]:
        assert lib.nt_multiply_mod(u64(int(a)), u64(int(b)), u64(int(m)), u64(0)) == int(r)
    for b, e, m, r in kats["power_mod"]:
        assert lib.nt_power_mod(u64(int(b)), u64(int(e)), u64(int(m))) == int(r)
    for r, d, m, expect in kats["is_primitive_root"]:
        assert lib.nt_is_primitive_root(u64(int(r)), u64(int(d)), u64(int(m))) == expect
    for a, m, r in kats["inverse_mod"]:
        assert lib.nt_inverse_mod(u64(int(a)), u64(int(m))) == int(r)
    counts = {k: len(v) for k, v in kats.items()}
    assert counts["multiply_mod"] == 10 and counts["power_mod"] == 6, counts
    assert counts["is_primitive_root"] == 6 and counts["inverse_mod"] == 3, counts
    return kats


class _RefTables(ctypes.Structure):
    # struct vkhel_ntt_tables (include/priv/ntt_tables.h:6-15)
    _fields_ = [("n", ctypes.c_uint64), ("q", ctypes.c_uint64), ("w", ctypes.c_uint64),
                ("roots", ctypes.POINTER(ctypes.c_uint64)),
                ("inv_roots", ctypes.POINTER(ctypes.c_uint64)),
                ("roots_shoup", ctypes.POINTER(ctypes.c_uint64)),
                ("inv_roots_shoup", ctypes.POINTER(ctypes.c_uint64))]


def reference_tables():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvkhelref.so"))
    lib.vkhel_ntt_tables_create.restype = ctypes.POINTER(_RefTables)
    lib.vkhel_ntt_tables_create.argtypes = [ctypes.c_uint64] * 3
    sets = [
        (4, 113, 18),
        (16, 2251799813685313, 110968848420801),
        # n = 4096, 16384, 65536 with the first primes = 1 (mod 2n) below 2^60
        # and w = x^((q-1)/2n) for the smallest x giving w^n = -1.
        (4096, 1152921504606830593, 431606828070683274),
        (16384, 1152921504606748673, 641000223749548346),
        (65536, 1152921504606584833, None),
        # the top of the modulus range (2^62 <= q < 2^63): the first such
        # primes below 2^63 (at n = 256 the reference's Barrett products
        # overflow there, so its "powers" of w are not w^i) and above 2^62,
        # and a degree past 2^18
        (256, _ntt_prime(256, 1 << 63, down=True), None),
        (4096, _ntt_prime(4096, 1 << 63, down=True), None),
        (16384, _ntt_prime(16384, 1 << 62, down=False), None),
        (1 << 20, _ntt_prime(1 << 20, 1 << 60, down=True), None),
        # the smallest degree, a 31-bit prime, the largest one-launch degree,
        # a degree past 2^20, and a w that is not a primitive 2n-th root (its
        # inverse table comes from the reference's per-entry extended Euclid)
        (2, 17, 4),
        (8192, _ntt_prime(8192, 1 << 31, down=True), None),
        (1 << 17, _ntt_prime(1 << 17, 1 << 60, down=True), None),
        (1 << 22, _ntt_prime(1 << 22, 1 << 60, down=True), None),
        (16, 2251799813685313, 3),
    ]
    out = []
    for n, q, w in sets:
        if w is None:  # exact arithmetic (the reference's own powers overflow at 63 bits)
            w = workloads.root_for(n, q)
        t = lib.vkhel_ntt_tables_create(n, q, w).contents
        arrays = {k: [getattr(t, k)[i] for i in range(n)]
                  for k in ("roots", "inv_roots", "roots_shoup", "inv_roots_shoup")}
        rec = {"n": str(n), "q": str(q), "w": str(w)}
        for k, v in arrays.items():
            raw = b"".join(x.to_bytes(8, "little") for x in v)
            rec[k + "_sha256"] = hashlib.sha256(raw).hexdigest()
            if n <= 64:
                rec[k] = [str(x) for x in v]
        out.append(rec)
    return out


def _ntt_prime(n, bound, down):
    """The first prime q = 1 (mod 2n) below (down) or above `bound`."""
    if down:
        return workloads.ntt_primes(n, 1, bound=bound)[0]
    q = (bound // (2 * n)) * (2 * n) + 1
    while not workloads.is_prime(q):
        q += 2 * n
    return q


def main():
    if not os.path.isdir(REF):
        sys.exit(f"reference checkout not found at {REF}")
    build_ref()
    passed, ops = vector_cases()
    with open(os.path.join(HERE, "reference_vectors.json"), "w") as f:
        json.dump({"source": "test/vector.c (lolzballs/vkhel), replayed on the CPU oracle; "
                             "the program's own assertions passed for: " + ", ".join(passed),
                   "ops": ops}, f, indent=1)
    with open(os.path.join(HERE, "reference_numbers.json"), "w") as f:
        json.dump({"source": "literals of test/numbers.c and test/ntt.c (lolzballs/vkhel), "
                             "checked against the reference's numbers.c",
                   "kats": number_kats()}, f, indent=1)
    with open(os.path.join(HERE, "reference_tables.json"), "w") as f:
        json.dump({"source": "src/ntt_tables.c (lolzballs/vkhel) built from source",
                   "tables": reference_tables()}, f, indent=1)
    print(f"{len(ops)} vector ops, tests passed: {passed}")


if __name__ == "__main__":
    main()
