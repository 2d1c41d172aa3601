"""Twiddle tables generated on the device equal the reference's host tables.

For q < 2^61 and a primitive 2n-th root w < q the library builds the device
tables with a kernel (w^i = w^(hi 2^lb) w^lo from two short power tables,
inverses by index, Shoup factors by 128/64 division) instead of uploading the
host arrays.  Every word must equal the host construction, which itself is
pinned to the reference's table digests (reference_tables.json).  Other
moduli and roots keep the host upload; their device copy must match too.
"""
import hashlib

import numpy as np
import pytest

from conftest import load_golden
from vkhel_gb300 import workloads

pytestmark = pytest.mark.gpu

KEYS = ("roots", "inv_roots", "roots_shoup", "inv_roots_shoup")


def _check(vk, ctx, n, q, w):
    t = vk.NttTables(n, q, w)
    dev = t.device_arrays(ctx)
    host = t.arrays()
    for k in KEYS:
        np.testing.assert_array_equal(dev[k], host[k], err_msg=f"{k} n={n} q={q} w={w}")
    return dev


@pytest.mark.parametrize("log_n", [1, 2, 4, 7, 10, 13, 14, 15, 17, 18])
@pytest.mark.parametrize("bits", [20, 30, 50, 60, 61])
def test_device_tables_equal_host_tables(vk, ctx, log_n, bits):
    n = 1 << log_n
    qs = workloads.ntt_primes(n, 1, bound=1 << bits)
    if not qs:
        pytest.skip("no prime q = 1 mod 2n below the bound")
    q = qs[0]
    _check(vk, ctx, n, q, workloads.root_for(n, q))


@pytest.mark.parametrize("rec", load_golden("reference_tables.json")["tables"], ids=lambda r: f"n{r['n']}")
def test_device_tables_match_reference_digests(vk, ctx, rec):
    dev = _check(vk, ctx, int(rec["n"]), int(rec["q"]), int(rec["w"]))
    for k in KEYS:
        assert hashlib.sha256(dev[k].astype("<u8").tobytes()).hexdigest() == rec[k + "_sha256"], k


def test_host_upload_cases_match(vk, ctx):
    n = 1024
    q62 = workloads.ntt_primes(n, 1, bound=1 << 62)[0]
    _check(vk, ctx, n, q62, workloads.root_for(n, q62))          # 62-bit modulus
    q = workloads.ntt_primes(n, 1)[0]
    w = workloads.root_for(n, q)
    _check(vk, ctx, n, q, w * w % q)                               # not a primitive 2n-th root
    _check(vk, ctx, n, q, w + q)                                   # root not reduced below q
    _check(vk, ctx, 1, q, w)                                       # n = 1


def test_device_tables_drive_exact_transforms(vk, ctx, oracle):
    for log_n in (12, 16):
        n = 1 << log_n
        q = workloads.ntt_primes(n, 1, bound=1 << 61)[0]
        w = workloads.root_for(n, q)
        t = vk.NttTables(n, q, w)
        rng = np.random.default_rng(log_n)
        a_h, b_h = workloads.uniform(rng, q, n), workloads.uniform(rng, q, n)
        a, b, c = vk.Vector(ctx, a_h), vk.Vector(ctx, b_h), vk.Vector(ctx, n)
        vk.polymul(a, b, c, t)
        np.testing.assert_array_equal(c.download(), oracle.polymul(a_h, b_h, n, q, w)[0])
