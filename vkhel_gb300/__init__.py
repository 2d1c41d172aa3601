"""vkhel_gb300: Python host mirror of the vkhel C API on GB300.

The product is ``libvkhel.so`` (C host layer + sm_103a CUDA kernels, built by
``vkhel_gb300.build``).  This module binds it with ctypes and mirrors the
reference's API objects one to one:

    reference (include/vkhel/vkhel.h)      here
    vkhel_ctx_create / _destroy            Context()
    vkhel_ntt_tables_create / _destroy     NttTables(n, q, w)
    vkhel_vector_create / create2 / ...    Vector(ctx, length, zero=True)
    vkhel_vector_elemfma / elemmod / ...   Vector methods and module functions

Operations are synchronous like the reference's.  Errors that the reference
turns into assert() aborts raise VkhelError here, carrying the library's
status code and message.  There is no fallback: if the library is missing,
importing ``lib()`` raises.
"""
import atexit
import ctypes
import os
import weakref

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libvkhel.so")

u64 = ctypes.c_uint64
u32 = ctypes.c_uint32
vp = ctypes.c_void_p
P64 = ctypes.POINTER(ctypes.c_uint64)

# (name, restype, argtypes) for every exported function of include/vkhel/*.h
_SIGNATURES = [
    ("vkhel_ctx_create", vp, []),
    ("vkhel_ctx_destroy", None, [vp]),
    ("vkhel_ntt_tables_create", vp, [u64, u64, u64]),
    ("vkhel_ntt_tables_destroy", None, [vp]),
    ("vkhel_vector_create", vp, [vp, u64]),
    ("vkhel_vector_create2", vp, [vp, u64, ctypes.c_bool]),
    ("vkhel_vector_destroy", None, [vp]),
    ("vkhel_vector_dup", vp, [vp]),
    ("vkhel_vector_copy_from_host", None, [vp, vp]),
    ("vkhel_vector_map", None, [vp, ctypes.POINTER(vp), ctypes.c_size_t]),
    ("vkhel_vector_unmap", None, [vp]),
    ("vkhel_vector_elemfma", None, [vp, vp, vp, u64, u64]),
    ("vkhel_vector_elemmod", None, [vp, vp, u64, u64]),
    ("vkhel_vector_elemmul", None, [vp, vp, vp, u64]),
    ("vkhel_vector_elemgtadd", None, [vp, vp, u64, u64]),
    ("vkhel_vector_elemgtsub", None, [vp, vp, u64, u64, u64]),
    ("vkhel_vector_forward_transform", None, [vp, vp, vp]),
    ("vkhel_vector_inverse_transform", None, [vp, vp, vp]),
    # extensions
    ("vkhel_ctx_last_error", ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t]),
    ("vkhel_ctx_clear_error", None, [vp]),
    ("vkhel_ctx_set_budget", ctypes.c_int, [vp, u64]),
    ("vkhel_ctx_bytes_in_use", u64, [vp]),
    ("vkhel_ctx_stream", vp, [vp]),
    ("vkhel_ctx_sync", ctypes.c_int, [vp]),
    ("vkhel_ctx_sm_count", ctypes.c_int, [vp]),
    ("vkhel_launch_count", u64, []),
    ("vkhel_measure_int_peak", ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("vkhel_vector_length", u64, [vp]),
    ("vkhel_vector_device_ptr", vp, [vp]),
    ("vkhel_vector_upload", ctypes.c_int, [vp, vp, u64]),
    ("vkhel_vector_download", ctypes.c_int, [vp, vp, u64]),
    ("vkhel_vector_upload_async", ctypes.c_int, [vp, vp, u64]),
    ("vkhel_vector_download_async", ctypes.c_int, [vp, vp, u64]),
    ("vkhel_vector_dbgprint", None, [vp]),
    ("vkhel_ntt_tables_copy", ctypes.c_int, [vp, vp, vp, vp, vp]),
    ("vkhel_ntt_tables_dbgprint", None, [vp]),
    ("vkhel_ntt_tables_device_copy", ctypes.c_int, [vp, vp, vp, vp, vp, vp]),
    ("vkhel_vector_elemfma_canonical", None, [vp, vp, vp, u64, u64]),
    ("vkhel_vector_polymul", ctypes.c_int, [vp, vp, vp, vp]),
    ("vkhel_vector_polymul_noalloc", ctypes.c_int, [vp, vp, vp, vp]),
    ("vkhel_vector_polymul_ntt", ctypes.c_int, [vp, vp, vp, vp]),
    ("vkhel_ctx_set_async", ctypes.c_int, [vp, ctypes.c_int]),
    ("vkhel_vector_polymul_lift", ctypes.c_int, [vp, vp, vp, vp, vp, u32]),
    ("vkhel_vector_inverse_transform_lift", ctypes.c_int, [vp, vp, vp, vp, u32]),
    ("vkhel_batch_create", vp, [vp]),
    ("vkhel_batch_add_polymul", ctypes.c_int, [vp, ctypes.POINTER(vp), u32, vp, vp, vp]),
    ("vkhel_batch_add_polymul_raw", ctypes.c_int, [vp, ctypes.POINTER(vp), u32, vp, vp, vp]),
    ("vkhel_batch_add_polymul_ntt", ctypes.c_int, [vp, ctypes.POINTER(vp), u32, vp, vp, vp]),
    ("vkhel_batch_add_polymul_ntt_raw", ctypes.c_int, [vp, ctypes.POINTER(vp), u32, vp, vp, vp]),
    ("vkhel_batch_add_polymul_lift", ctypes.c_int, [vp, ctypes.POINTER(vp), u32, vp, vp, vp, vp, u32]),
    ("vkhel_batch_add_transform", ctypes.c_int, [vp, ctypes.POINTER(vp), u32, vp, vp, u32, vp, u32]),
    ("vkhel_debug_fail_allocations", ctypes.c_int, [u64, u64]),
    ("vkhel_server_cancel", ctypes.c_int, [vp, ctypes.c_int64]),
    ("vkhel_elem_batch_create", vp, [vp]),
    ("vkhel_elem_batch_add", ctypes.c_int, [vp, u32, u64, u64, u64, vp, vp, vp]),
    ("vkhel_elem_batch_add_raw", ctypes.c_int, [vp, u32, u64, u64, u64, vp, vp, vp, u64]),
    ("vkhel_elem_batch_commit", ctypes.c_int, [vp, u32]),
    ("vkhel_elem_batch_launch", ctypes.c_int, [vp]),
    ("vkhel_elem_batch_run", ctypes.c_int, [vp]),
    ("vkhel_elem_batch_jobs", u32, [vp]),
    ("vkhel_elem_batch_destroy", None, [vp]),
    ("vkhel_batch_commit", ctypes.c_int, [vp, u32]),
    ("vkhel_batch_launch", ctypes.c_int, [vp]),
    ("vkhel_batch_run", ctypes.c_int, [vp]),
    ("vkhel_batch_jobs", u32, [vp]),
    ("vkhel_batch_kernels", u32, [vp]),
    ("vkhel_batch_destroy", None, [vp]),
    ("vkhel_tune_set", ctypes.c_int, [u32, u32, ctypes.c_int32]),
    ("vkhel_tune_get", ctypes.c_int, [u32, u32]),
    ("vkhel_tune_load", ctypes.c_int, [ctypes.c_char_p]),
    ("vkhel_server_create", vp, [vp]),
    ("vkhel_server_submit", ctypes.c_int64, [vp, ctypes.POINTER(vp), u32, vp, vp, vp]),
    ("vkhel_server_add_operand", ctypes.c_int64, [vp, ctypes.POINTER(vp), u32, vp, ctypes.c_int]),
    ("vkhel_server_submit_operand", ctypes.c_int64, [vp, ctypes.POINTER(vp), u32, vp, ctypes.c_int64, vp]),
    ("vkhel_server_remove_operand", ctypes.c_int, [vp, ctypes.c_int64]),
    ("vkhel_server_wait", ctypes.c_int, [vp, ctypes.c_int64, u32]),
    ("vkhel_server_stats", ctypes.c_int, [vp, vp]),
    ("vkhel_server_reset_stats", ctypes.c_int, [vp]),
    ("vkhel_server_destroy", None, [vp]),
]

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "OUT_OF_MEMORY", 3: "BUDGET", 4: "DEVICE",
          5: "NO_DEVICE", 6: "TIMEOUT", 7: "CANCELLED", 8: "UNSUPPORTED"}
BATCH_GRAPH = 1

_lib = None
_live_contexts = weakref.WeakSet()


@atexit.register
def _close_all_contexts():
    # Destroy contexts (and their vectors) while the interpreter and the CUDA
    # runtime are fully alive, instead of in arbitrary finalizer order.
    for c in list(_live_contexts):
        try:
            c.close()
        except Exception:
            pass


class VkhelError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"vkhel {STATUS.get(code, code)}: {msg}")
        self.code = code
        self.msg = msg


def lib(path=None):
    """Load libvkhel.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("VKHEL_LIB", LIB_PATH)
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} missing: build it with `python -m vkhel_gb300.build`")
    L = ctypes.CDLL(p)
    for name, res, args in _SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = L
    return L


def last_error(ctx_ptr=None):
    buf = ctypes.create_string_buffer(256)
    code = lib().vkhel_ctx_last_error(ctx_ptr, buf, 256)
    return code, buf.value.decode(errors="replace")


def _check_ctx(ctx_ptr):
    code, msg = last_error(ctx_ptr)
    if code:
        lib().vkhel_ctx_clear_error(ctx_ptr)
        raise VkhelError(code, msg)


def _status(ctx_ptr, code):
    if code:
        _, msg = last_error(ctx_ptr)
        lib().vkhel_ctx_clear_error(ctx_ptr)
        raise VkhelError(code, msg)


def _as_u64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64))


class Context:
    """vkhel_ctx: one CUDA device, stream and device pool."""

    def __init__(self):
        L = lib()
        L.vkhel_ctx_clear_error(None)
        self.ptr = L.vkhel_ctx_create()
        if not self.ptr:
            code, msg = last_error(None)
            raise VkhelError(code or 5, msg)
        self._children = weakref.WeakSet()
        _live_contexts.add(self)

    def close(self):
        if self.ptr:
            for ch in list(self._children):
                ch.close()
            lib().vkhel_ctx_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return lib().vkhel_ctx_stream(self.ptr)

    @property
    def sm_count(self):
        return lib().vkhel_ctx_sm_count(self.ptr)

    def sync(self):
        _status(self.ptr, lib().vkhel_ctx_sync(self.ptr))

    def set_budget(self, nbytes):
        _status(self.ptr, lib().vkhel_ctx_set_budget(self.ptr, int(nbytes)))

    def set_async(self, on=True):
        """vkhel_ctx_set_async: single calls return once their kernels are enqueued."""
        _status(self.ptr, lib().vkhel_ctx_set_async(self.ptr, 1 if on else 0))

    @property
    def bytes_in_use(self):
        return lib().vkhel_ctx_bytes_in_use(self.ptr)

    def vector(self, length_or_data, zero=True):
        return Vector(self, length_or_data, zero)

    def measure_int_peak(self):
        """(butterflies/s, IMAD/s) of this GPU, measured now."""
        b, i = ctypes.c_double(), ctypes.c_double()
        _status(self.ptr, lib().vkhel_measure_int_peak(self.ptr, ctypes.byref(b), ctypes.byref(i)))
        return b.value, i.value


class NttTables:
    """vkhel_ntt_tables for degree n, modulus q, primitive 2n-th root w."""

    def __init__(self, n, q, w):
        L = lib()
        L.vkhel_ctx_clear_error(None)
        self.n, self.q, self.w = int(n), int(q), int(w)
        self.ptr = L.vkhel_ntt_tables_create(self.n, self.q, self.w)
        if not self.ptr:
            code, msg = last_error(None)
            raise VkhelError(code or 1, msg)

    def arrays(self):
        out = [np.zeros(self.n, dtype=np.uint64) for _ in range(4)]
        lib().vkhel_ntt_tables_copy(self.ptr, *[o.ctypes.data for o in out])
        return dict(zip(("roots", "inv_roots", "roots_shoup", "inv_roots_shoup"), out))

    def device_arrays(self, ctx):
        """The context's device copy (generated on the GPU when q < 2^61)."""
        out = [np.zeros(self.n, dtype=np.uint64) for _ in range(4)]
        _status(ctx.ptr, lib().vkhel_ntt_tables_device_copy(ctx.ptr, self.ptr, *[o.ctypes.data for o in out]))
        return dict(zip(("roots", "inv_roots", "roots_shoup", "inv_roots_shoup"), out))

    def close(self):
        if self.ptr:
            lib().vkhel_ntt_tables_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Vector:
    """vkhel_vector: `length` device-resident uint64 words."""

    def __init__(self, ctx, length_or_data, zero=True):
        L = lib()
        self.ctx = ctx
        data = None
        if np.ndim(length_or_data) > 0:
            data = _as_u64(length_or_data)
            length = data.size
            zero = False
        else:
            length = int(length_or_data)
        self.ptr = L.vkhel_vector_create2(ctx.ptr, length, bool(zero))
        if not self.ptr:
            _check_ctx(ctx.ptr)
            raise VkhelError(2, "vector_create failed")
        self.length = length
        ctx._children.add(self)
        if data is not None:
            self.upload(data)

    @classmethod
    def _wrap(cls, ctx, ptr, length):
        v = cls.__new__(cls)
        v.ctx, v.ptr, v.length = ctx, ptr, length
        ctx._children.add(v)
        return v

    def close(self):
        # A vector outliving its context was freed with the context's pool.
        if getattr(self, "ptr", None) and getattr(self.ctx, "ptr", None):
            lib().vkhel_vector_destroy(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_ptr(self):
        return lib().vkhel_vector_device_ptr(self.ptr)

    def upload(self, data):
        data = _as_u64(data)
        _status(self.ctx.ptr, lib().vkhel_vector_upload(self.ptr, data.ctypes.data, data.size))

    def upload_async(self, host, count=None):
        """vkhel_vector_upload_async: enqueue a copy of `count` words (all of
        `host` by default) from a uint64 numpy array or a torch tensor; `host`
        must stay alive and unchanged until the context is synchronized."""
        count = (host.size if isinstance(host, np.ndarray) else host.numel()) if count is None else count
        _status(self.ctx.ptr, lib().vkhel_vector_upload_async(self.ptr, _ptr(host), int(count)))

    def download_async(self, host, count=None):
        """vkhel_vector_download_async into `host` (uint64 numpy array or torch
        tensor); the words are there once the context is synchronized."""
        count = (host.size if isinstance(host, np.ndarray) else host.numel()) if count is None else count
        _status(self.ctx.ptr, lib().vkhel_vector_download_async(self.ptr, _ptr(host), int(count)))

    def copy_from_host(self, data):
        data = _as_u64(data)
        assert data.size >= self.length
        lib().vkhel_vector_copy_from_host(self.ptr, data.ctypes.data)
        _check_ctx(self.ctx.ptr)

    def download(self, count=None):
        count = self.length if count is None else count
        out = np.empty(count, dtype=np.uint64)
        _status(self.ctx.ptr, lib().vkhel_vector_download(self.ptr, out.ctypes.data, count))
        return out

    def map_read(self, size=None):
        """Contents through vkhel_vector_map / unmap (the reference's path)."""
        size = self.length * 8 if size is None else size
        p = vp()
        L = lib()
        L.vkhel_vector_map(self.ptr, ctypes.byref(p), size)
        _check_ctx(self.ctx.ptr)
        out = np.ctypeslib.as_array(ctypes.cast(p, P64), shape=(self.length,)).copy() if self.length else \
            np.empty(0, np.uint64)
        L.vkhel_vector_unmap(self.ptr)
        _check_ctx(self.ctx.ptr)
        return out

    def dup(self):
        p = lib().vkhel_vector_dup(self.ptr)
        if not p:
            _check_ctx(self.ctx.ptr)
        return Vector._wrap(self.ctx, p, self.length)


def _op(name, *args):
    getattr(lib(), name)(*[a.ptr if isinstance(a, (Vector, NttTables)) else a for a in args])
    ctx = next(a.ctx for a in args if isinstance(a, Vector))
    _check_ctx(ctx.ptr)


def elemfma(a, b, res, multiplier, mod): _op("vkhel_vector_elemfma", a, b, res, int(multiplier), int(mod))
def elemfma_canonical(a, b, res, multiplier, mod): _op("vkhel_vector_elemfma_canonical", a, b, res, int(multiplier), int(mod))
def elemmod(a, res, mod, q): _op("vkhel_vector_elemmod", a, res, int(mod), int(q))
def elemmul(a, b, res, mod): _op("vkhel_vector_elemmul", a, b, res, int(mod))
def elemgtadd(a, res, bound, diff): _op("vkhel_vector_elemgtadd", a, res, int(bound), int(diff))
def elemgtsub(a, res, bound, diff, mod): _op("vkhel_vector_elemgtsub", a, res, int(bound), int(diff), int(mod))
def forward_transform(a, res, tables): _op("vkhel_vector_forward_transform", a, res, tables)
def inverse_transform(a, res, tables): _op("vkhel_vector_inverse_transform", a, res, tables)


def polymul(a, b, res, tables):
    _status(res.ctx.ptr, lib().vkhel_vector_polymul(a.ptr, b.ptr, res.ptr, tables.ptr))


def polymul_ntt(a, b_ntt, res, tables):
    """vkhel_vector_polymul_ntt: the product with b given as NTT(b) (a forward transform's output)."""
    _status(res.ctx.ptr, lib().vkhel_vector_polymul_ntt(a.ptr, b_ntt.ptr, res.ptr, tables.ptr))


def polymul_noalloc(a, b, res, tables):
    """vkhel_vector_polymul_noalloc: same product, scratch in a static device array."""
    _status(res.ctx.ptr, lib().vkhel_vector_polymul_noalloc(a.ptr, b.ptr, res.ptr, tables.ptr))


# Centred-lift epilogue steps (struct vkhel_lift_step): the reference's
# element-wise ops applied in order after the inverse transform.
LIFT_ELEMMOD, LIFT_ELEMGTSUB, LIFT_ELEMGTADD = 1, 2, 3
MAX_LIFT_STEPS = 4


class LiftStep(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint32), ("p0", ctypes.c_uint64), ("p1", ctypes.c_uint64), ("p2", ctypes.c_uint64)]


def lift_steps(steps):
    """[("elemmod", mod, q), ("elemgtsub", bound, diff, mod), ("elemgtadd", bound, diff)] -> C array.

    elemmod with q = 0 takes q from the transform's tables (each limb's, in a batch)."""
    ops = {"elemmod": LIFT_ELEMMOD, "elemgtsub": LIFT_ELEMGTSUB, "elemgtadd": LIFT_ELEMGTADD}
    arr = (LiftStep * max(1, len(steps)))()
    for i, st in enumerate(steps):
        op = ops.get(st[0], st[0])
        params = [int(x) for x in st[1:]] + [0, 0, 0]
        arr[i] = LiftStep(int(op), *params[:3])
    return arr, len(steps)


def polymul_lift(a, b, res, tables, steps):
    arr, n = lift_steps(steps)
    _status(res.ctx.ptr, lib().vkhel_vector_polymul_lift(a.ptr, b.ptr, res.ptr, tables.ptr, ctypes.addressof(arr), n))


def inverse_transform_lift(a, res, tables, steps):
    arr, n = lift_steps(steps)
    _status(res.ctx.ptr, lib().vkhel_vector_inverse_transform_lift(a.ptr, res.ptr, tables.ptr,
                                                                   ctypes.addressof(arr), n))


def launch_count():
    return lib().vkhel_launch_count()


def fail_allocations(skip, count):
    """Test fault injection: after `skip` device allocations the next `count` fail."""
    lib().vkhel_debug_fail_allocations(int(skip), int(count))


class Batch:
    """vkhel_batch: a committed list of limb products launched as one unit."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.ptr = lib().vkhel_batch_create(ctx.ptr)
        if not self.ptr:
            _check_ctx(ctx.ptr)
        self._keep = []
        ctx._children.add(self)

    def add_polymul(self, tables, a, b, c, lift=None, b_ntt=False):
        """Limb products of a and b into c; b_ntt=True: b holds NTT(b) of every limb."""
        arr = (vp * len(tables))(*[t.ptr for t in tables])
        self._keep.append((tables, a, b, c))  # the batch reads and writes them at every launch
        if b_ntt:
            if lift:
                raise ValueError("b_ntt has no lift form")
            if isinstance(a, Vector):
                code = lib().vkhel_batch_add_polymul_ntt(self.ptr, arr, len(tables), a.ptr, b.ptr, c.ptr)
            else:
                code = lib().vkhel_batch_add_polymul_ntt_raw(self.ptr, arr, len(tables), int(a), int(b), int(c))
        elif lift:
            steps, n = lift_steps(lift)
            code = lib().vkhel_batch_add_polymul_lift(self.ptr, arr, len(tables), a.ptr, b.ptr, c.ptr,
                                                      ctypes.addressof(steps), n)
        elif isinstance(a, Vector):
            code = lib().vkhel_batch_add_polymul(self.ptr, arr, len(tables), a.ptr, b.ptr, c.ptr)
        else:  # raw device pointers
            code = lib().vkhel_batch_add_polymul_raw(self.ptr, arr, len(tables), int(a), int(b), int(c))
        _status(self.ctx.ptr, code)

    def add_transform(self, tables, inp, out, inverse=False, lift=None):
        """Forward (or inverse, optionally with a lift) transform of every limb of inp into out."""
        arr = (vp * len(tables))(*[t.ptr for t in tables])
        self._keep.append((tables, inp, out))
        steps, n = lift_steps(lift or [])
        _status(self.ctx.ptr, lib().vkhel_batch_add_transform(self.ptr, arr, len(tables), inp.ptr, out.ptr,
                                                              1 if inverse else 0, ctypes.addressof(steps), n))

    def commit(self, graph=True):
        _status(self.ctx.ptr, lib().vkhel_batch_commit(self.ptr, BATCH_GRAPH if graph else 0))

    def launch(self):
        _status(self.ctx.ptr, lib().vkhel_batch_launch(self.ptr))

    def run(self):
        _status(self.ctx.ptr, lib().vkhel_batch_run(self.ptr))

    @property
    def jobs(self):
        return lib().vkhel_batch_jobs(self.ptr)

    @property
    def kernels(self):
        return lib().vkhel_batch_kernels(self.ptr)

    def close(self):
        if getattr(self, "ptr", None) and getattr(self.ctx, "ptr", None):
            lib().vkhel_batch_destroy(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


ELEM_OPS = {"elemfma": 1, "elemfma_canonical": 2, "elemmul": 3, "elemmulconst": 4, "elemmod": 5,
            "elemgtadd": 6, "elemgtsub": 7}


class ElemBatch:
    """vkhel_elem_batch: independent element-wise jobs of ragged lengths in one launch."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.ptr = lib().vkhel_elem_batch_create(ctx.ptr)
        if not self.ptr:
            _check_ctx(ctx.ptr)
        self._keep = []
        ctx._children.add(self)

    def add(self, op, a, b, res, *params):
        """op name (elemfma, elemmod, ...) with the single call's parameters in order."""
        p = [int(x) for x in params] + [0, 0, 0]
        code = ELEM_OPS.get(op, op)
        if isinstance(res, Vector):
            self._keep.append((a, b, res))
            rc = lib().vkhel_elem_batch_add(self.ptr, code, p[0], p[1], p[2], a.ptr, b.ptr if b is not None else None,
                                            res.ptr)
        else:  # (device pointer, length) for res; device pointers (or vectors) for a and b
            ptr, n = res
            dp = lambda x: None if x is None else (x.device_ptr if isinstance(x, Vector) else int(x))
            self._keep.append((a, b))
            rc = lib().vkhel_elem_batch_add_raw(self.ptr, code, p[0], p[1], p[2], dp(a), dp(b), int(ptr), int(n))
        _status(self.ctx.ptr, rc)

    def commit(self, graph=True):
        _status(self.ctx.ptr, lib().vkhel_elem_batch_commit(self.ptr, BATCH_GRAPH if graph else 0))

    def launch(self):
        _status(self.ctx.ptr, lib().vkhel_elem_batch_launch(self.ptr))

    def run(self):
        _status(self.ctx.ptr, lib().vkhel_elem_batch_run(self.ptr))

    @property
    def jobs(self):
        return lib().vkhel_elem_batch_jobs(self.ptr)

    def close(self):
        if getattr(self, "ptr", None) and getattr(self.ctx, "ptr", None):
            lib().vkhel_elem_batch_destroy(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerConfig(ctypes.Structure):
    _fields_ = [("device_budget", ctypes.c_uint64), ("max_batch_limbs", ctypes.c_uint32),
                ("max_inflight_batches", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("limbs", ctypes.c_uint64), ("span_s", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Server:
    """vkhel_server: continuous batching of polynomial-multiply requests.

    submit() takes NttTables per limb and host uint64 arrays (limb-major,
    limbs * n words); the arrays are kept referenced until wait() returns.
    """

    def __init__(self, device_budget=0, max_batch_limbs=0, max_inflight_batches=0):
        cfg = ServerConfig(int(device_budget), int(max_batch_limbs), int(max_inflight_batches))
        lib().vkhel_ctx_clear_error(None)
        self.ptr = lib().vkhel_server_create(ctypes.byref(cfg))
        if not self.ptr:
            code, msg = last_error(None)
            raise VkhelError(code or 4, msg)
        self._pending = {}
        self._operands = {}

    def submit(self, tables, a, b, c):
        arr = (vp * len(tables))(*[t.ptr for t in tables])
        rid = lib().vkhel_server_submit(self.ptr, arr, len(tables), _ptr(a), _ptr(b), _ptr(c))
        if rid < 0:
            code, msg = last_error(None)
            lib().vkhel_ctx_clear_error(None)
            raise VkhelError(-rid, msg)
        self._pending[rid] = (tables, a, b, c)
        return rid

    def add_operand(self, tables, b, is_ntt=False):
        """Keep b (or NTT(b), is_ntt=True) resident on the server; returns the operand id."""
        arr = (vp * len(tables))(*[t.ptr for t in tables])
        oid = lib().vkhel_server_add_operand(self.ptr, arr, len(tables), _ptr(b), 1 if is_ntt else 0)
        if oid < 0:
            code, msg = last_error(None)
            lib().vkhel_ctx_clear_error(None)
            raise VkhelError(-oid, msg)
        self._operands[oid] = tables
        return oid

    def submit_operand(self, tables, a, operand, c):
        """A request c = a * b with b the resident operand `operand`."""
        arr = (vp * len(tables))(*[t.ptr for t in tables])
        rid = lib().vkhel_server_submit_operand(self.ptr, arr, len(tables), _ptr(a), int(operand), _ptr(c))
        if rid < 0:
            code, msg = last_error(None)
            lib().vkhel_ctx_clear_error(None)
            raise VkhelError(-rid, msg)
        self._pending[rid] = (tables, a, c)
        return rid

    def remove_operand(self, operand):
        st = lib().vkhel_server_remove_operand(self.ptr, int(operand))
        if st:
            code, msg = last_error(None)
            lib().vkhel_ctx_clear_error(None)
            raise VkhelError(st, msg)
        self._operands.pop(operand, None)

    def cancel(self, rid):
        """Cancel a request still queued; returns its status code (0 = cancelled)."""
        st = lib().vkhel_server_cancel(self.ptr, rid)
        if st:
            lib().vkhel_ctx_clear_error(None)
        return st

    def wait(self, rid, timeout_ms=60000):
        st = lib().vkhel_server_wait(self.ptr, rid, int(timeout_ms))
        if st != 6:  # not a timeout: the id is collected
            self._pending.pop(rid, None)
        return st

    def stats(self):
        s = ServerStats()
        lib().vkhel_server_stats(self.ptr, ctypes.byref(s))
        return s.as_dict()

    def reset_stats(self):
        lib().vkhel_server_reset_stats(self.ptr)

    def close(self):
        if getattr(self, "ptr", None):
            lib().vkhel_server_destroy(self.ptr)
            self.ptr = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ptr(x):
    """Host address of a numpy array or a torch tensor (pinned or not)."""
    if isinstance(x, np.ndarray):
        assert x.dtype == np.uint64 and x.flags.c_contiguous
        return x.ctypes.data
    return x.data_ptr()
