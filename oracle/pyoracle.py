"""ctypes binding of the CPU oracle (oracle/oracle.c) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg,
always to compare against or as the timed CPU baseline, never as part of the product.
``load()`` builds oracle/_build/liboracle.so with make if it is missing.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

u64 = ctypes.c_uint64
sz = ctypes.c_size_t
vp = ctypes.c_void_p

_SIGS = {
    "orc_bitlen": (u64, [u64]),
    "orc_shoup_factor": (u64, [u64, u64]),
    "orc_barrett_mu": (u64, [u64]),
    "orc_mulmod": (u64, [u64, u64, u64]),
    "orc_powmod": (u64, [u64, u64, u64]),
    "orc_is_primitive_root": (ctypes.c_bool, [u64, u64, u64]),
    "orc_invmod": (u64, [u64, u64]),
    "orc_ntt_tables": (None, [u64, u64, u64, vp, vp, vp, vp]),
    "orc_elemmul": (None, [vp, vp, vp, sz, u64]),
    "orc_elemmulconst": (None, [vp, vp, sz, u64, u64]),
    "orc_elemfma": (None, [vp, vp, vp, sz, u64, u64]),
    "orc_elemfma_canonical": (None, [vp, vp, vp, sz, u64, u64]),
    "orc_elemgtsub": (None, [vp, vp, sz, u64, u64, u64]),
    "orc_elemgtadd": (None, [vp, vp, sz, u64, u64]),
    "orc_elemmodbytwo": (None, [vp, vp, sz, u64]),
    "orc_elemmod": (None, [vp, vp, sz, u64, u64]),
    "orc_ntt_forward": (ctypes.c_int, [vp, u64, u64, vp, vp]),
    "orc_ntt_inverse": (ctypes.c_int, [vp, u64, u64, vp, vp]),
    "orc_polymul": (ctypes.c_int, [vp, vp, vp, u64, u64, u64]),
    "orc_negacyclic_schoolbook": (None, [vp, vp, vp, u64, u64]),
    "orc_polymul_batch": (ctypes.c_int, [vp, vp, vp, sz, sz, u64, vp, vp, vp, sz, ctypes.c_int]),
    "orc_polymul_batch_tables": (ctypes.c_int, [vp, vp, vp, sz, sz, u64, vp, vp, vp, ctypes.c_int]),
}


def _u64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64))


class Oracle:
    def __init__(self, path=LIB):
        self.L = ctypes.CDLL(path)
        for k, (res, args) in _SIGS.items():
            f = getattr(self.L, k)
            f.restype, f.argtypes = res, args

    # scalars
    def mulmod(self, a, b, q): return self.L.orc_mulmod(a, b, q)
    def powmod(self, a, e, q): return self.L.orc_powmod(a, e, q)
    def invmod(self, a, q): return self.L.orc_invmod(a, q)
    def is_primitive_root(self, r, d, q): return self.L.orc_is_primitive_root(r, d, q)
    def shoup(self, f, q): return self.L.orc_shoup_factor(f, q)

    def tables(self, n, q, w):
        t = [np.zeros(n, np.uint64) for _ in range(4)]
        self.L.orc_ntt_tables(n, q, w, *[x.ctypes.data for x in t])
        return dict(zip(("roots", "inv_roots", "roots_shoup", "inv_roots_shoup"), t))

    def _un(self, fn, a, *params):
        a = _u64(a)
        r = np.zeros_like(a)
        getattr(self.L, fn)(a.ctypes.data, r.ctypes.data, a.size, *params)
        return r

    def _bin(self, fn, a, b, *params):
        a, b = _u64(a), _u64(b)
        r = np.zeros_like(a)
        getattr(self.L, fn)(a.ctypes.data, b.ctypes.data, r.ctypes.data, a.size, *params)
        return r

    def elemmul(self, a, b, mod): return self._bin("orc_elemmul", a, b, mod)
    def elemfma(self, a, b, m, mod): return self._bin("orc_elemfma", a, b, m, mod)
    def elemfma_canonical(self, a, b, m, mod): return self._bin("orc_elemfma_canonical", a, b, m, mod)
    def elemmulconst(self, a, c, mod): return self._un("orc_elemmulconst", a, c, mod)
    def elemgtsub(self, a, bound, diff, mod): return self._un("orc_elemgtsub", a, bound, diff, mod)
    def elemgtadd(self, a, bound, diff): return self._un("orc_elemgtadd", a, bound, diff)
    def elemmod(self, a, mod, q): return self._un("orc_elemmod", a, mod, q)

    def forward(self, a, n, q, w, tables=None):
        t = tables or self.tables(n, q, w)
        d = _u64(a)[:n].copy()
        st = self.L.orc_ntt_forward(d.ctypes.data, n, q, t["roots"].ctypes.data, t["roots_shoup"].ctypes.data)
        return d, st

    def inverse(self, a, n, q, w, tables=None):
        t = tables or self.tables(n, q, w)
        d = _u64(a)[:n].copy()
        st = self.L.orc_ntt_inverse(d.ctypes.data, n, q, t["inv_roots"].ctypes.data,
                                    t["inv_roots_shoup"].ctypes.data)
        return d, st

    def polymul(self, a, b, n, q, w):
        a, b = _u64(a), _u64(b)
        c = np.zeros(n, np.uint64)
        st = self.L.orc_polymul(a.ctypes.data, b.ctypes.data, c.ctypes.data, n, q, w)
        return c, st

    def schoolbook(self, a, b, n, q):
        a, b = _u64(a), _u64(b)
        c = np.zeros(n, np.uint64)
        self.L.orc_negacyclic_schoolbook(a.ctypes.data, b.ctypes.data, c.ctypes.data, n, q)
        return c

    def batch_tables(self, n, qs, ws):
        """The primes' tables for polymul_batch, built once: (len(qs), 4 n) uint64."""
        t = np.zeros((len(qs), 4 * n), np.uint64)
        for p, (q, w) in enumerate(zip(qs, ws)):
            row = t[p]
            self.L.orc_ntt_tables(n, int(q), int(w), *[row[i * n:].ctypes.data for i in range(4)])
        return t

    def polymul_batch(self, a, b, n, qs, ws, prime_idx, threads=0, tables=None):
        """a, b: (count, n) uint64.  Returns (c, threads used).  With `tables`
        from batch_tables(n, qs, ws) the tables are not rebuilt per call."""
        a, b = _u64(a), _u64(b)
        count = a.shape[0]
        c = np.zeros_like(a)
        qs, ws = _u64(qs), _u64(ws)
        pi = np.ascontiguousarray(np.asarray(prime_idx, dtype=np.uint32))
        if tables is not None:
            t = np.ascontiguousarray(tables, dtype=np.uint64)
            used = self.L.orc_polymul_batch_tables(a.ctypes.data, b.ctypes.data, c.ctypes.data, count, n, n,
                                                   qs.ctypes.data, t.ctypes.data, pi.ctypes.data, threads)
        else:
            used = self.L.orc_polymul_batch(a.ctypes.data, b.ctypes.data, c.ctypes.data, count, n, n,
                                            qs.ctypes.data, ws.ctypes.data, pi.ctypes.data, qs.size, threads)
        return c, used


def reference_dir():
    """The reference checkout's location as oracle/Makefile resolves it
    (VKHEL_REF overrides it), or None where it is absent (GPU machines)."""
    try:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                           capture_output=True, text=True, timeout=30)
    except (OSError, subprocess.SubprocessError):
        return None
    d = r.stdout.strip()
    return d if r.returncode == 0 and d and os.path.isdir(os.path.join(d, "src")) else None


_oracle = None


def load():
    global _oracle
    if _oracle is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "oracle.c")):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        _oracle = Oracle()
    return _oracle
