"""ctypes binding of libbsgpu.so (the C ABI declared in include/bsg.h).

This module is the Python side of the drop-in boundary: it loads the
in-tree library and fails loudly when it is missing -- there is no CPU
fallback.  Pointer arguments accept numpy arrays (host), objects with a
``data_ptr()`` method such as torch CUDA tensors (device), or raw ints.
"""
from __future__ import annotations

import atexit
import ctypes
import os
import sys
import weakref

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libbsgpu.so")

# flags (include/bsg.h)
HOST_PTRS = 0x000
DEVICE_PTRS = 0x001
ASYNC = 0x002
MODE_FAST = 0x000
MODE_SFU_REF = 0x010
MODE_LIBM_REF = 0x020
NO_GRAPH = 0x100
NUM_RUNS = 100
MAX_ERR_BUCKETS = 32

MODES = {"fast": MODE_FAST, "sfu_ref": MODE_SFU_REF, "libm_ref": MODE_LIBM_REF}

STATUS = {
    0: "BSG_OK", -1: "BSG_ERR_INVALID_ARG", -2: "BSG_ERR_NO_DEVICE",
    -3: "BSG_ERR_CUDA", -4: "BSG_ERR_OUT_OF_MEMORY", -5: "BSG_ERR_CAPACITY",
    -6: "BSG_ERR_MISALIGNED", -7: "BSG_ERR_TIMEOUT", -8: "BSG_ERR_BUDGET",
    -9: "BSG_ERR_CANCELLED", -10: "BSG_ERR_NOT_SUPPORTED", -11: "BSG_ERR_STATE",
}


class BsgError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


class Segment(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_uint64), ("len", ctypes.c_uint64)]


class ErrBucket(ctypes.Structure):
    _fields_ = [("count", ctypes.c_uint64), ("max_abs", ctypes.c_double),
                ("sum_sq_abs", ctypes.c_double), ("max_rel", ctypes.c_double),
                ("max_price", ctypes.c_double)]


class Tune(ctypes.Structure):
    _fields_ = [("vec_per_thread", ctypes.c_int), ("block", ctypes.c_int),
                ("blocks_per_sm", ctypes.c_int), ("load_path", ctypes.c_int),
                ("pdl", ctypes.c_int), ("resident_32nds", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("budget_bytes", ctypes.c_size_t),
                ("max_inflight", ctypes.c_int), ("max_batch_options", ctypes.c_size_t),
                ("max_batch_requests", ctypes.c_int), ("plain", ctypes.c_int),
                ("flags", ctypes.c_uint), ("batch_timeout_s", ctypes.c_double),
                ("fused", ctypes.c_int), ("persistent_blocks", ctypes.c_int),
                ("persistent_window", ctypes.c_int)]


class Request(ctypes.Structure):
    _fields_ = [("sptprice", ctypes.c_void_p), ("strike", ctypes.c_void_p),
                ("rate", ctypes.c_void_p), ("volatility", ctypes.c_void_p),
                ("otime", ctypes.c_void_p), ("otype", ctypes.c_void_p),
                ("prices", ctypes.c_void_p), ("n", ctypes.c_size_t)]


class ServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in (
        "submitted", "completed", "cancelled", "failed", "batches", "kernel_launches",
        "options_priced", "max_batch_requests_seen", "queued", "inflight_requests")]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class TraceConfig(ctypes.Structure):
    _fields_ = [("rate_per_s", ctypes.c_double), ("duration_s", ctypes.c_double),
                ("min_n", ctypes.c_size_t), ("max_n", ctypes.c_size_t),
                ("seed", ctypes.c_uint64),
                ("sptprice", ctypes.c_void_p), ("strike", ctypes.c_void_p),
                ("rate", ctypes.c_void_p), ("volatility", ctypes.c_void_p),
                ("otime", ctypes.c_void_p), ("otype", ctypes.c_void_p),
                ("prices", ctypes.c_void_p), ("pool_n", ctypes.c_size_t),
                ("drain_timeout_s", ctypes.c_double)]


class TraceResult(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("options", ctypes.c_uint64),
                ("wall_s", ctypes.c_double), ("options_per_s", ctypes.c_double),
                ("requests_per_s", ctypes.c_double), ("p50_s", ctypes.c_double),
                ("p99_s", ctypes.c_double), ("p999_s", ctypes.c_double),
                ("max_s", ctypes.c_double), ("mean_s", ctypes.c_double),
                ("mean_batch_requests", ctypes.c_double), ("batches", ctypes.c_uint64),
                ("late_submit_max_s", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BookC(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("sptprice", ctypes.c_void_p),
                ("strike", ctypes.c_void_p), ("rate", ctypes.c_void_p),
                ("volatility", ctypes.c_void_p), ("otime", ctypes.c_void_p),
                ("otype", ctypes.c_void_p), ("dgrefval", ctypes.c_void_p),
                ("mem_", ctypes.c_void_p)]


class BatchTune(ctypes.Structure):
    _fields_ = [("tile_options", ctypes.c_uint64), ("blocks_per_sm", ctypes.c_int)]

    def as_dict(self):
        return {"tile_options": int(self.tile_options), "blocks_per_sm": int(self.blocks_per_sm)}


class SwaptionC(ctypes.Structure):
    """bsg_swaption (include/bsg.h)."""
    _fields_ = [("strike", ctypes.c_double), ("compounding", ctypes.c_double),
                ("maturity", ctypes.c_double), ("tenor", ctypes.c_double),
                ("payment_interval", ctypes.c_double), ("years", ctypes.c_double),
                ("n_steps", ctypes.c_int), ("n_factors", ctypes.c_int),
                ("yield_", ctypes.c_void_p), ("factors", ctypes.c_void_p),
                ("seed", ctypes.c_uint64)]


# Every symbol the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_I = ctypes.c_int
_U = ctypes.c_uint
SIGNATURES = {
    "bsg_create": (_I, [ctypes.POINTER(_P), _I, _SZ]),
    "bsg_destroy": (None, [_P]),
    "bsg_strerror": (ctypes.c_char_p, [_I]),
    "bsg_last_error": (ctypes.c_char_p, [_P]),
    "bsg_stream": (_P, [_P]),
    "bsg_synchronize": (_I, [_P]),
    "bsg_kernel_launches": (ctypes.c_uint64, [_P]),
    "bsg_host_alloc": (_P, [_SZ]),
    "bsg_host_free": (None, [_P]),
    "bsg_price_soa": (_I, [_P] + [_P] * 7 + [_SZ, _I, _U]),
    "bsg_BlkSchlsEqEuroNoDiv": (_I, [_P, _I] + [_P] * 6 + [ctypes.c_float]),
    "bsg_price_fp64": (_I, [_P] + [_P] * 7 + [_SZ, _U]),
    "bsg_price_soa_f64": (_I, [_P] + [_P] * 7 + [_SZ, _I, _U]),
    "bsg_price_batch": (_I, [_P] + [_P] * 7 + [_SZ, ctypes.POINTER(Segment), _SZ, _I, _U]),
    "bsg_autotune_batch": (_I, [_P] + [_P] * 7 + [_SZ, ctypes.POINTER(Segment), _SZ,
                                                  ctypes.POINTER(BatchTune)]),
    "bsg_get_batch_tune": (_I, [_P, ctypes.POINTER(BatchTune)]),
    "bsg_set_batch_tune": (_I, [_P, ctypes.POINTER(BatchTune)]),
    "bsg_price_books_plain": (_I, [_P] + [_P] * 7 + [_SZ, ctypes.POINTER(Segment), _SZ, _I, _U]),
    "bsg_price_batch_noalloc": (_I, [_P] * 7 + [_SZ, ctypes.POINTER(Segment), _SZ, _P, _U]),
    "bsg_error_report": (_I, [_P] + [_P] * 7 + [_SZ, _P, _I, ctypes.c_double, ctypes.POINTER(ErrBucket)]),
    "bsg_server_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(ServerConfig)]),
    "bsg_server_destroy": (None, [_P]),
    "bsg_server_register": (_I, [_P, _P, _SZ]),
    "bsg_server_submit": (_I, [_P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "bsg_server_wait": (_I, [_P, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "bsg_server_cancel": (_I, [_P, ctypes.c_uint64]),
    "bsg_server_pause": (_I, [_P, _I]),
    "bsg_server_get_stats": (_I, [_P, ctypes.POINTER(ServerStats)]),
    "bsg_serve_trace": (_I, [ctypes.POINTER(ServerConfig), ctypes.POINTER(TraceConfig),
                             ctypes.POINTER(TraceResult), _P, _SZ]),
    "bsg_read_parsec": (_I, [ctypes.c_char_p, _I, ctypes.POINTER(BookC)]),
    "bsg_parse_parsec": (_I, [ctypes.c_char_p, _SZ, _I, ctypes.POINTER(BookC)]),
    "bsg_book_free": (None, [ctypes.POINTER(BookC)]),
    "bsg_write_parsec_prices": (_I, [ctypes.c_char_p, _P, _SZ, _I]),
    "bsg_format_prices": (_I, [_P, _SZ, _I, ctypes.POINTER(ctypes.c_void_p),
                               ctypes.POINTER(ctypes.c_size_t)]),
    "bsg_text_free": (None, [ctypes.c_void_p]),
    "bsg_write_parsec_input": (_I, [ctypes.c_char_p, ctypes.POINTER(BookC), _I]),
    "bsg_write_soa": (_I, [ctypes.c_char_p, ctypes.POINTER(BookC)]),
    "bsg_read_soa": (_I, [ctypes.c_char_p, ctypes.POINTER(BookC)]),
    "bsg_autotune": (_I, [_P, _SZ, ctypes.POINTER(Tune)]),
    "bsg_selftest_wait_timeout": (_I, [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "bsg_selftest_guard": (_I, [_P]),
    "bsg_get_tune": (_I, [_P, ctypes.POINTER(Tune)]),
    "bsg_set_tune": (_I, [_P, ctypes.POINTER(Tune)]),
    "bsg_price_swaptions": (_I, [_P, ctypes.POINTER(SwaptionC), _SZ, ctypes.c_uint64, _P, _P]),
    "bsg_swaption_normals": (_I, [_P, _P, _SZ, _P]),
    "bsg_HJM_Swaption_Blocking": (_I, [_P] + [ctypes.c_double] * 5 + [_I, _I, ctypes.c_double,
                                                                       _P, _P, ctypes.c_long,
                                                                       ctypes.c_long, _I, _I]),
}

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libbsgpu.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python -m p3arsec_gb300.build); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(x) -> int:
    """Address of a numpy array, a tensor-like with data_ptr(), or an int."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    raise TypeError(f"cannot take the address of {type(x)!r}")


def _check(lib, ctx, st):
    if st != 0:
        msg = lib.bsg_last_error(ctx).decode() if ctx else ""
        if not msg:
            msg = lib.bsg_strerror(st).decode()
        raise BsgError(st, msg)


# Contexts and servers still open when the interpreter exits are closed by
# an atexit hook, while the CUDA runtime and every library that shares the
# device are still loaded; a finaliser that runs later, during interpreter
# teardown, leaves the handle to the process exit instead of calling into a
# runtime that may already be shutting down.
_live = weakref.WeakSet()


@atexit.register
def _close_live():
    for obj in list(_live):
        try:
            obj.close()
        except Exception:  # noqa: BLE001 -- best effort at exit
            pass


class Context:
    """One GPU pricing context (bsg_ctx): a device, a stream, resident buffers."""

    def __init__(self, device: int = 0, max_options: int = 1 << 20):
        self.lib = load()
        h = _P()
        st = self.lib.bsg_create(ctypes.byref(h), device, max_options)
        if st != 0:
            raise BsgError(st, self.lib.bsg_strerror(st).decode())
        self.h = h
        self.device = device
        self.max_options = max_options
        _live.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.lib.bsg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.bsg_stream(self.h) or 0)

    def synchronize(self):
        """bsg_synchronize: waits for everything enqueued (pipelined calls too)."""
        _check(self.lib, self.h, self.lib.bsg_synchronize(self.h))

    @property
    def launches(self) -> int:
        return int(self.lib.bsg_kernel_launches(self.h))

    # ------------------------------------------------------------ pricing
    def price_soa(self, s, k, r, v, t, otype, prices, n=None, num_runs=1,
                  mode="fast", device=False, asynchronous=False, graph=True):
        """bsg_price_soa over host numpy arrays or device pointers."""
        if n is None:
            n = len(s)
        flags = MODES[mode] | (DEVICE_PTRS if device else HOST_PTRS)
        if asynchronous:
            flags |= ASYNC
        if not graph:
            flags |= NO_GRAPH
        if not device:
            for a, dt in ((s, np.float32), (k, np.float32), (r, np.float32), (v, np.float32),
                          (t, np.float32), (otype, np.int32), (prices, np.float32)):
                if not (isinstance(a, np.ndarray) and a.dtype == dt and a.flags.c_contiguous
                        and a.shape[0] >= n):
                    raise TypeError("host arrays must be C-contiguous float32 (otype int32) of length >= n")
        st = self.lib.bsg_price_soa(self.h, ptr(s), ptr(k), ptr(r), ptr(v), ptr(t), ptr(otype),
                                    ptr(prices), n, num_runs, flags)
        _check(self.lib, self.h, st)
        return prices

    def price_book(self, book, num_runs=1, mode="fast"):
        """Prices a host ``books.Book``; returns a new float32 array."""
        out = np.empty(len(book), dtype=np.float32)
        self.price_soa(*book.arrays(), out, n=len(book), num_runs=num_runs, mode=mode)
        return out

    def price_fp64(self, s, k, r, v, t, otype, out, n=None, device=False):
        if n is None:
            n = len(s)
        flags = DEVICE_PTRS if device else HOST_PTRS
        st = self.lib.bsg_price_fp64(self.h, ptr(s), ptr(k), ptr(r), ptr(v), ptr(t), ptr(otype),
                                     ptr(out), n, flags)
        _check(self.lib, self.h, st)
        return out

    def price_soa_f64(self, s, k, r, v, t, otype, prices, n=None, num_runs=1, device=False,
                      asynchronous=False):
        """FP64 product mode: double arrays in, double prices out."""
        if n is None:
            n = len(s)
        flags = (DEVICE_PTRS if device else HOST_PTRS) | (ASYNC if asynchronous else 0)
        st = self.lib.bsg_price_soa_f64(self.h, ptr(s), ptr(k), ptr(r), ptr(v), ptr(t),
                                        ptr(otype), ptr(prices), n, num_runs, flags)
        _check(self.lib, self.h, st)
        return prices

    def price_batch(self, pool, prices, pool_len, segments, num_runs=1, mode="fast",
                    plain=False, asynchronous=False, graph=True):
        """Batched books over a device pool (pool = 6 device pointers)."""
        segs = (Segment * max(len(segments), 1))()
        for i, (o, l) in enumerate(segments):
            segs[i].offset = int(o)
            segs[i].len = int(l)
        flags = MODES[mode] | DEVICE_PTRS
        if asynchronous:
            flags |= ASYNC
        if not graph:
            flags |= NO_GRAPH
        fn = self.lib.bsg_price_books_plain if plain else self.lib.bsg_price_batch
        st = fn(self.h, *[ptr(x) for x in pool], ptr(prices), pool_len, segs, len(segments),
                num_runs, flags)
        _check(self.lib, self.h, st)

    def autotune_batch(self, pool, prices, pool_len, segments) -> dict:
        segs = (Segment * max(len(segments), 1))()
        for i, (o, l) in enumerate(segments):
            segs[i].offset = int(o)
            segs[i].len = int(l)
        t = BatchTune()
        st = self.lib.bsg_autotune_batch(self.h, *[ptr(x) for x in pool], ptr(prices), pool_len,
                                         segs, len(segments), ctypes.byref(t))
        _check(self.lib, self.h, st)
        return t.as_dict()

    def set_batch_tune(self, tile_options=8192, blocks_per_sm=0):
        t = BatchTune(tile_options, blocks_per_sm)
        _check(self.lib, self.h, self.lib.bsg_set_batch_tune(self.h, ctypes.byref(t)))

    def get_batch_tune(self) -> dict:
        t = BatchTune()
        _check(self.lib, self.h, self.lib.bsg_get_batch_tune(self.h, ctypes.byref(t)))
        return t.as_dict()

    def error_report(self, pool, prices, n, edges, rel_floor=1e-3):
        """bsg_error_report over device arrays; returns a list of dicts."""
        edges = np.ascontiguousarray(edges, dtype=np.float64)
        nb = len(edges) - 1
        out = (ErrBucket * nb)()
        st = self.lib.bsg_error_report(self.h, *[ptr(x) for x in pool], ptr(prices), n,
                                       ptr(edges), nb, rel_floor, out)
        _check(self.lib, self.h, st)
        res = []
        for i in range(nb):
            b = out[i]
            res.append({"d1_lo": float(edges[i]), "d1_hi": float(edges[i + 1]),
                        "count": int(b.count), "max_abs": b.max_abs,
                        "rms_abs": (b.sum_sq_abs / b.count) ** 0.5 if b.count else 0.0,
                        "sum_sq_abs": b.sum_sq_abs, "max_rel": b.max_rel,
                        "max_price": b.max_price})
        return res

    # ------------------------------------------------------------- tuning
    def autotune(self, n: int) -> dict:
        t = Tune()
        st = self.lib.bsg_autotune(self.h, n, ctypes.byref(t))
        _check(self.lib, self.h, st)
        return t.as_dict()

    def selftest_wait_timeout(self, limit_s: float = 0.05):
        """Makes the staged kernel's bounded waits expire; returns (status, seconds)."""
        el = ctypes.c_double()
        st = self.lib.bsg_selftest_wait_timeout(self.h, limit_s, ctypes.byref(el))
        return st, el.value

    def selftest_guard(self):
        """Plants one overwritten debug guard word; returns (status, message)."""
        st = self.lib.bsg_selftest_guard(self.h)
        return st, self.lib.bsg_last_error(self.h).decode()

    def get_tune(self) -> dict:
        t = Tune()
        _check(self.lib, self.h, self.lib.bsg_get_tune(self.h, ctypes.byref(t)))
        return t.as_dict()

    # ---------------------------------------------------------- swaptions
    def price_swaptions(self, swaptions, trials: int):
        """bsg_price_swaptions over p3arsec_gb300.swaptions.Swaption objects;
        returns (prices, standard errors) as float64 arrays."""
        arr, keep = swaption_structs(swaptions)
        n = len(swaptions)
        price = np.empty(n)
        err = np.empty(n)
        st = self.lib.bsg_price_swaptions(self.h, arr, n, trials, ptr(price), ptr(err))
        _check(self.lib, self.h, st)
        return price, err

    def swaption_normals(self, words):
        """bsg_swaption_normals: the swaption kernel's normal pairs of the
        uint32 words (4 per pair); returns float64 z of 2 per pair."""
        w = np.ascontiguousarray(words, dtype=np.uint32)
        if w.size % 4:
            raise ValueError("4 words per pair")
        z = np.empty(w.size // 2)
        st = self.lib.bsg_swaption_normals(self.h, ptr(w), w.size // 4, ptr(z))
        _check(self.lib, self.h, st)
        return z

    def set_tune(self, vec_per_thread=1, block=256, blocks_per_sm=0, load_path=0, pdl=0,
                 resident_32nds=0):
        t = Tune(vec_per_thread, block, blocks_per_sm, load_path, pdl, resident_32nds)
        _check(self.lib, self.h, self.lib.bsg_set_tune(self.h, ctypes.byref(t)))


class Server:
    """bsg_server: the continuous-batching request loop (see include/bsg.h)."""

    def __init__(self, device=0, budget_bytes=64 << 30, max_inflight=4, max_batch_options=0,
                 max_batch_requests=0, plain=False, mode="fast", batch_timeout_s=30.0,
                 fused=True, persistent=False, persistent_blocks=0, persistent_window=0):
        self.lib = load()
        self.cfg = ServerConfig(device, budget_bytes, max_inflight, max_batch_options,
                                max_batch_requests, 1 if plain else 0, MODES[mode],
                                batch_timeout_s, 2 if persistent else (1 if fused else 0),
                                persistent_blocks, persistent_window)
        h = _P()
        st = self.lib.bsg_server_create(ctypes.byref(h), ctypes.byref(self.cfg))
        if st != 0:
            raise BsgError(st, self.lib.bsg_strerror(st).decode())
        self.h = h
        _live.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.lib.bsg_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def register(self, arr):
        """Pin/register a host array (numpy) for batched requests."""
        st = self.lib.bsg_server_register(self.h, ptr(arr), arr.nbytes)
        if st != 0:
            raise BsgError(st, self.lib.bsg_strerror(st).decode())

    def submit(self, s, k, r, v, t, otype, prices, n=None) -> int:
        if n is None:
            n = len(s)
        req = Request(ptr(s), ptr(k), ptr(r), ptr(v), ptr(t), ptr(otype), ptr(prices), n)
        rid = ctypes.c_uint64()
        st = self.lib.bsg_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid))
        if st != 0:
            raise BsgError(st, self.lib.bsg_strerror(st).decode())
        return int(rid.value)

    def wait(self, rid: int, timeout_s: float = -1.0):
        """Returns (status, latency_s); status BSG_ERR_TIMEOUT leaves it pending."""
        lat = ctypes.c_double(float("nan"))
        st = self.lib.bsg_server_wait(self.h, rid, timeout_s, ctypes.byref(lat))
        return st, lat.value

    def cancel(self, rid: int) -> int:
        return self.lib.bsg_server_cancel(self.h, rid)

    def pause(self, paused: bool = True):
        self.lib.bsg_server_pause(self.h, 1 if paused else 0)

    def stats(self) -> dict:
        x = ServerStats()
        self.lib.bsg_server_get_stats(self.h, ctypes.byref(x))
        return x.as_dict()


def serve_trace(host_pool, prices, rate_per_s, duration_s, min_n=16, max_n=1 << 20, seed=1,
                device=0, budget_bytes=64 << 30, max_inflight=4, plain=False, mode="fast",
                max_batch_options=0, max_batch_requests=0, drain_timeout_s=60.0,
                latencies=None, fused=True, persistent=False, persistent_blocks=0,
                persistent_window=0):
    """bsg_serve_trace over a host pool (6 arrays) and a prices array."""
    lib = load()
    cfg = ServerConfig(device, budget_bytes, max_inflight, max_batch_options, max_batch_requests,
                       1 if plain else 0, MODES[mode], 30.0,
                       2 if persistent else (1 if fused else 0), persistent_blocks,
                       persistent_window)
    n = len(host_pool[0])
    tc = TraceConfig(rate_per_s, duration_s, min_n, max_n, seed, *[ptr(a) for a in host_pool],
                     ptr(prices), n, drain_timeout_s)
    res = TraceResult()
    cap = 0 if latencies is None else len(latencies)
    st = lib.bsg_serve_trace(ctypes.byref(cfg), ctypes.byref(tc), ctypes.byref(res),
                             ptr(latencies) if latencies is not None else None, cap)
    if st != 0:
        raise BsgError(st, lib.bsg_strerror(st).decode())
    return res.as_dict()


def swaption_structs(swaptions):
    """bsg_swaption array for p3arsec_gb300.swaptions.Swaption objects, and the
    numpy arrays it points into (keep them alive while the array is used)."""
    keep, arr = [], (SwaptionC * max(len(swaptions), 1))()
    for i, w in enumerate(swaptions):
        y = np.ascontiguousarray(w.yield_curve, dtype=np.float64)
        f = np.ascontiguousarray(w.factors, dtype=np.float64)
        keep += [y, f]
        arr[i] = SwaptionC(w.strike, w.compounding, w.maturity, w.tenor, w.payment_interval,
                           w.years, w.n_steps, w.n_factors, y.ctypes.data, f.ctypes.data, w.seed)
    return arr, keep


def HJM_Swaption_Blocking(w, trials: int):
    """The reference's per-swaption call shape (bsg_HJM_Swaption_Blocking):
    returns (status, price, standard error); status 1 = success."""
    lib = load()
    y = np.ascontiguousarray(w.yield_curve, dtype=np.float64)
    rows = [np.ascontiguousarray(r, dtype=np.float64) for r in w.factors]
    pp = (ctypes.c_void_p * len(rows))(*[r.ctypes.data for r in rows])
    out = np.zeros(2)
    st = lib.bsg_HJM_Swaption_Blocking(ptr(out), w.strike, w.compounding, w.maturity, w.tenor,
                                       w.payment_interval, w.n_steps, w.n_factors, w.years,
                                       ptr(y), ctypes.cast(pp, ctypes.c_void_p), w.seed, trials,
                                       16, 0)
    return st, float(out[0]), float(out[1])


NOALLOC_MAX_SEGMENTS = 4096


def price_batch_noalloc(pool, prices, pool_len, segments, stream=0, asynchronous=False):
    """bsg_price_batch_noalloc: batched books with no allocation (device pool
    pointers, current device, caller's stream).  Returns the status code."""
    lib = load()
    segs = (Segment * max(len(segments), 1))()
    for i, (o, l) in enumerate(segments):
        segs[i].offset = int(o)
        segs[i].len = int(l)
    flags = DEVICE_PTRS | (ASYNC if asynchronous else 0)
    return lib.bsg_price_batch_noalloc(*[ptr(x) for x in pool], ptr(prices), pool_len, segs,
                                       len(segments), stream, flags)


# ------------------------------------------------------------------ file I/O
def _book_from_c(b: BookC):
    from .books import Book
    n = int(b.n)

    def arr(addr, dt):
        if n == 0:
            return np.zeros(0, dtype=dt)
        raw = (ctypes.c_char * (4 * n)).from_address(addr)
        return np.frombuffer(raw, dtype=dt).copy()
    book = Book(arr(b.sptprice, np.float32), arr(b.strike, np.float32), arr(b.rate, np.float32),
                arr(b.volatility, np.float32), arr(b.otime, np.float32), arr(b.otype, np.int32))
    return book, arr(b.dgrefval, np.float32)


def read_parsec(path, nthreads: int = 0):
    """bsg_read_parsec: (Book, dgrefval) from a PARSEC input file."""
    lib = load()
    b = BookC()
    st = lib.bsg_read_parsec(os.fsencode(path), nthreads, ctypes.byref(b))
    if st != 0:
        raise BsgError(st, f"cannot read {path}")
    try:
        return _book_from_c(b)
    finally:
        lib.bsg_book_free(ctypes.byref(b))


def parse_parsec(text: bytes, nthreads: int = 0):
    lib = load()
    b = BookC()
    st = lib.bsg_parse_parsec(text, len(text), nthreads, ctypes.byref(b))
    if st != 0:
        raise BsgError(st, "cannot parse PARSEC text")
    try:
        return _book_from_c(b)
    finally:
        lib.bsg_book_free(ctypes.byref(b))


def format_prices(prices, nthreads: int = 0) -> bytes:
    """bsg_format_prices: the reference's output file as bytes."""
    lib = load()
    p = np.ascontiguousarray(prices, dtype=np.float32)
    text = ctypes.c_void_p()
    ln = ctypes.c_size_t()
    st = lib.bsg_format_prices(ptr(p), len(p), nthreads, ctypes.byref(text), ctypes.byref(ln))
    if st != 0:
        raise BsgError(st, "format failed")
    try:
        return ctypes.string_at(text.value, ln.value)
    finally:
        lib.bsg_text_free(text)


def write_parsec_prices(path, prices, nthreads: int = 0):
    lib = load()
    p = np.ascontiguousarray(prices, dtype=np.float32)
    st = lib.bsg_write_parsec_prices(os.fsencode(path), ptr(p), len(p), nthreads)
    if st != 0:
        raise BsgError(st, f"cannot write {path}")


def write_parsec_input(path, book, dgrefval=None, nthreads: int = 0):
    """bsg_write_parsec_input: a PARSEC input file from a Book (parallel)."""
    lib = load()
    n = len(book)
    arrs = [np.ascontiguousarray(a) for a in book.arrays()]
    dg = None if dgrefval is None else np.ascontiguousarray(dgrefval, np.float32)
    b = BookC(n, *[ptr(a) for a in arrs], ptr(dg) if dg is not None else None, None)
    st = lib.bsg_write_parsec_input(os.fsencode(path), ctypes.byref(b), nthreads)
    if st != 0:
        raise BsgError(st, f"cannot write {path}")


def write_soa(path, book, dgrefval=None):
    lib = load()
    n = len(book)
    arrs = [np.ascontiguousarray(a) for a in book.arrays()]
    dg = np.zeros(n, np.float32) if dgrefval is None else np.ascontiguousarray(dgrefval, np.float32)
    b = BookC(n, *[ptr(a) for a in arrs], ptr(dg), None)
    st = lib.bsg_write_soa(os.fsencode(path), ctypes.byref(b))
    if st != 0:
        raise BsgError(st, f"cannot write {path}")


def read_soa(path):
    lib = load()
    b = BookC()
    st = lib.bsg_read_soa(os.fsencode(path), ctypes.byref(b))
    if st != 0:
        raise BsgError(st, f"cannot read {path}")
    try:
        return _book_from_c(b)
    finally:
        lib.bsg_book_free(ctypes.byref(b))


def BlkSchlsEqEuroNoDiv(OptionPrice, numOptions, sptprice, strike, rate, volatility,
                        time, otype, timet=0.0):
    """The reference's batch entry point (blackscholes.simd.c:221-223) on the GPU.

    Prices ``numOptions`` options once into ``OptionPrice`` (host float32
    arrays; otype int32).  ``timet`` is unused, as in the reference.
    """
    lib = load()
    st = lib.bsg_BlkSchlsEqEuroNoDiv(ptr(OptionPrice), numOptions, ptr(sptprice), ptr(strike),
                                     ptr(rate), ptr(volatility), ptr(time), ptr(otype), timet)
    if st != 0:
        raise BsgError(st, lib.bsg_strerror(st).decode())
    return OptionPrice
