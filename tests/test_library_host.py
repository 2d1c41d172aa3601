"""libvkhel.so without a GPU: symbols, host tables, error paths.

These run in the CPU suite.  They load the product library (its C host layer
works without a device), check that it exports exactly the functions declared
in include/vkhel/*.h and nothing else (the reference's version script makes
every vkhel_* global and everything else local, vkhel.syms:1-6), compare the
host twiddle tables it builds with the reference's own tables, and exercise
the reported-error paths that replace the reference's assert() aborts.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden, u64
from vkhel_gb300 import workloads

HEADERS = [os.path.join(ROOT, "include", "vkhel", h) for h in ("vkhel.h", "vkhel_ext.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(vkhel_[a-z0-9_]+)\s*\(", src))
    return names


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if l.strip()}


def test_exports_exactly_the_declared_api(vk):
    from vkhel_gb300 import LIB_PATH
    decl = declared_functions()
    exp = exported_symbols(LIB_PATH)
    # all 18 functions of the reference header are among them
    ref18 = {"vkhel_ctx_create", "vkhel_ctx_destroy", "vkhel_ntt_tables_create", "vkhel_ntt_tables_destroy",
             "vkhel_vector_create", "vkhel_vector_create2", "vkhel_vector_destroy", "vkhel_vector_dup",
             "vkhel_vector_copy_from_host", "vkhel_vector_map", "vkhel_vector_unmap", "vkhel_vector_elemfma",
             "vkhel_vector_elemmod", "vkhel_vector_elemmul", "vkhel_vector_elemgtadd", "vkhel_vector_elemgtsub",
             "vkhel_vector_forward_transform", "vkhel_vector_inverse_transform"}
    assert ref18 <= decl
    missing = decl - exp
    assert not missing, f"declared but not exported: {sorted(missing)}"
    extra = {s for s in exp if not s.startswith("vkhel_")}
    assert not extra, f"non-vkhel symbols exported: {sorted(extra)[:10]}"
    assert exp - decl == set(), f"exported but undeclared: {sorted(exp - decl)}"


def test_python_binding_covers_every_declared_function(vk):
    bound = {name for name, _, _ in vk._SIGNATURES}
    assert declared_functions() <= bound


@pytest.mark.parametrize("rec", load_golden("reference_tables.json")["tables"], ids=lambda r: f"n{r['n']}")
def test_host_tables_equal_reference_tables(vk, rec):
    import hashlib
    t = vk.NttTables(int(rec["n"]), int(rec["q"]), int(rec["w"]))
    for k, v in t.arrays().items():
        assert hashlib.sha256(v.astype("<u8").tobytes()).hexdigest() == rec[k + "_sha256"], k


@pytest.mark.parametrize("n,bits", [(2, 20), (8, 30), (256, 40), (4096, 61), (1024, 62), (256, 63), (4096, 63),
                                    (16384, 63)])
def test_host_tables_equal_oracle(vk, oracle, n, bits):
    q = workloads.ntt_primes(n, 1, bound=1 << bits)[0]
    w = workloads.root_for(n, q)
    got = vk.NttTables(n, q, w).arrays()
    ref = oracle.tables(n, q, w)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


def test_host_tables_non_primitive_root_uses_euclid(vk, oracle):
    # w = a non-primitive element: the inverse table must still equal the
    # reference's per-entry extended-Euclid inverses
    n, q = 16, 2251799813685313
    w = 3
    got = vk.NttTables(n, q, w).arrays()
    ref = oracle.tables(n, q, w)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.parametrize("n,q", [(0, 17), (3, 17), (12, 97), (4, 1), (4, 0)])
def test_tables_reject_invalid_parameters(vk, n, q):
    with pytest.raises(vk.VkhelError) as e:
        vk.NttTables(n, q, 1)
    assert e.value.code == 1


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_context_without_device_reports_no_device(vk):
    with pytest.raises(vk.VkhelError) as e:
        vk.Context()
    assert e.value.code == 5


def test_strict_mode_aborts_like_reference_assert():
    # VKHEL_STRICT=1 turns a failure into abort(), as the reference's assert()
    code = ("import vkhel_gb300 as v; L = v.lib(); L.vkhel_ntt_tables_create(3, 17, 1)")
    r = subprocess.run(["python", "-c", code], cwd=ROOT, env=dict(os.environ, VKHEL_STRICT="1"),
                       capture_output=True, text=True)
    assert r.returncode != 0 and "not a power of two" in r.stderr


def test_workload_prime_rule():
    assert workloads.ntt_primes(4096, 1) == [1152921504606830593]
    assert workloads.root_for(4096, 1152921504606830593) == 431606828070683274
    qs = workloads.ntt_primes(16384, 8)
    assert qs[0] == 1152921504606748673 and len(set(qs)) == 8
    assert all(q % (2 * 16384) == 1 and q < 1 << 60 and workloads.is_prime(q) for q in qs)
    for q in qs:
        w = workloads.root_for(16384, q)
        assert pow(w, 16384, q) == q - 1


def _flush_c_stdout():
    import ctypes
    ctypes.CDLL(None).fflush(None)


def test_tables_dbgprint_matches_reference_format(vk, oracle, capfd):
    # src/ntt_tables.c:46-63: header line, then the roots and the inverse roots
    n, q = 16, 2251799813685313
    w = 110968848420801
    t = vk.NttTables(n, q, w)
    vk.lib().vkhel_ntt_tables_dbgprint(t.ptr)
    _flush_c_stdout()
    out = capfd.readouterr().out
    ref = oracle.tables(n, q, w)
    expect = (f"ntt_tables: (n={n} q={q} w={w})\n"
              f"\troots_of_unity: {', '.join(str(int(x)) for x in ref['roots'])}\n"
              f"\tinv_roots_of_unity: {', '.join(str(int(x)) for x in ref['inv_roots'])}\n")
    assert out == expect


def test_tuning_table_parsing_and_overrides(vk, tmp_path):
    """The variant table: "family log_n variant" lines, '#' comments, lines
    that do not parse or name an unknown family / degree / a negative variant
    ignored; vkhel_tune_set / _get at run time; the committed GB300 table
    names a variant for every CTA-resident degree of the three kernel
    families and the concurrent-classes flag.  (Host only: no device.)"""
    L = vk.lib()
    table = os.path.join(ROOT, "vkhel_gb300", "tuning", "gb300.txt")
    saved = {(f, n): L.vkhel_tune_get(f, n) for f in range(4) for n in range(32)}
    try:
        t = tmp_path / "table.txt"
        t.write_text("# comment line\n0 14 1   # trailing comment\n1 13 2\nnot a line\n"
                     "9 10 1\n0 40 1\n2 12 -1\n2 11 1 extra\n")
        assert L.vkhel_tune_load(str(t).encode()) == 0
        assert L.vkhel_tune_get(0, 14) == 1 and L.vkhel_tune_get(1, 13) == 2 and L.vkhel_tune_get(2, 11) == 1
        assert L.vkhel_tune_get(2, 12) == saved[(2, 12)]       # negative variant ignored
        assert L.vkhel_tune_load(str(tmp_path / "missing.txt").encode()) != 0
        assert L.vkhel_tune_set(3, 1, 1) == 0 and L.vkhel_tune_get(3, 1) == 1
        assert L.vkhel_tune_set(4, 1, 1) != 0 and L.vkhel_tune_set(0, 32, 1) != 0 and L.vkhel_tune_set(0, 1, -1) != 0
        lib_clear_error = getattr(L, "vkhel_ctx_clear_error", None)
        if lib_clear_error:
            lib_clear_error(None)
        entries = set()
        buckets = set()
        for line in open(table):
            line = line.split("#")[0].split()
            if len(line) in (3, 4):
                entries.add((int(line[0]), int(line[1])))
                if len(line) == 4:
                    buckets.add((int(line[0]), int(line[1]), int(line[3])))
        for fam in (0, 1, 2):
            assert {(fam, n) for n in range(8, 15)} <= entries, f"family {fam} incomplete"
            assert {(fam, n, b) for n in range(8, 15) for b in range(4)} <= buckets, f"family {fam} buckets"
        assert (3, 0) in entries
        # a bucket field sets that job-count bucket only; vkhel_tune_get reads the many-jobs bucket (3)
        t.write_text("0 13 2\n0 13 1 0\n")
        assert L.vkhel_tune_load(str(t).encode()) == 0 and L.vkhel_tune_get(0, 13) == 2
        t.write_text("0 13 1 3\n0 13 0 9\n")
        assert L.vkhel_tune_load(str(t).encode()) == 0 and L.vkhel_tune_get(0, 13) == 1
    finally:
        for (f, n), v in saved.items():
            L.vkhel_tune_set(f, n, v)


def test_lazy_host_tables_under_concurrent_first_requests(vk, oracle):
    """Tables the device can generate (q < 2^61) build their host arrays only
    on first request, under a lock: eight threads asking for them at once
    (ctypes releases the GIL during the call) all get the oracle's arrays.
    Host only: no device."""
    import threading
    n = 1 << 14
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    ref = oracle.tables(n, q, w)
    for _ in range(3):  # fresh tables each round: the first request races
        t = vk.NttTables(n, q, w)
        results, go = [None] * 8, threading.Barrier(8)

        def worker(i):
            go.wait()
            results[i] = t.arrays()

        threads = [threading.Thread(target=worker, args=(i,)) for i in range(8)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        for r in results:
            for k, v in ref.items():
                np.testing.assert_array_equal(r[k], v, err_msg=k)
        t.close()
