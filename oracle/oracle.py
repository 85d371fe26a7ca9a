"""ctypes wrappers of the CPU oracle (TEST INFRASTRUCTURE ONLY).

* ``libbsoracle.so`` -- the C restatement of the reference's pricing path
  (bs_oracle.c; blackscholes.c:126-258 and the FastFlow map driver
  blackscholes.c:315-348), plus the FP64 same-formula oracle.  Built here and
  on any machine with gcc.
* ``_ref/libbsref.so`` -- the reference's own blackscholes.c compiled from its
  source tree (only where that tree is present).

The FP32 restatement is bit-identical to the reference on the same inputs
(pinned by tests/golden against outputs of the compiled reference).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libbsoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libbsref.so")
REF_SIMD_SO = {4: os.path.join(HERE, "_ref", "libbsref_simd4.so"),
               2: os.path.join(HERE, "_ref", "libbsref_simd2.so")}

_P = ctypes.c_void_p
_lib = None
_ref = None


def build(ref: bool = True) -> None:
    """make the restatement; and the reference (when its source tree, named
    by $P3ARSEC_REF as the Makefile says, exists -- else make skips it)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO) or (
                os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "bs_oracle.c"))):
            build(ref=False)
        L = ctypes.CDLL(ORACLE_SO)
        L.bso_cndf_ref.restype = ctypes.c_float
        L.bso_cndf_ref.argtypes = [ctypes.c_float]
        L.bso_price_ref.restype = ctypes.c_float
        L.bso_price_ref.argtypes = [ctypes.c_float] * 5 + [ctypes.c_int]
        L.bso_cndf_fp64.restype = ctypes.c_double
        L.bso_cndf_fp64.argtypes = [ctypes.c_double]
        L.bso_price_fp64.restype = ctypes.c_double
        L.bso_price_fp64.argtypes = [ctypes.c_double] * 5 + [ctypes.c_int]
        L.bso_d1_fp64.restype = ctypes.c_double
        L.bso_d1_fp64.argtypes = [ctypes.c_double] * 5
        L.bso_price_ref_soa.restype = None
        L.bso_price_ref_soa.argtypes = [ctypes.c_size_t] + [_P] * 7
        L.bso_price_ref_cr_soa.restype = None
        L.bso_price_ref_cr_soa.argtypes = [ctypes.c_size_t] + [_P] * 7
        L.bso_price_fp64_soa.restype = None
        L.bso_price_fp64_soa.argtypes = [ctypes.c_size_t] + [_P] * 7
        L.bso_price_fp64_soa_d.restype = None
        L.bso_price_fp64_soa_d.argtypes = [ctypes.c_size_t] + [_P] * 7
        L.bso_static_partition.restype = None
        L.bso_static_partition.argtypes = [ctypes.c_int64, ctypes.c_int, _P, _P]
        L.bso_read_parsec_fscanf.restype = ctypes.c_long
        L.bso_read_parsec_fscanf.argtypes = [ctypes.c_char_p, ctypes.c_size_t] + [_P] * 7
        L.bso_write_prices_fprintf.restype = ctypes.c_int
        L.bso_write_prices_fprintf.argtypes = [ctypes.c_char_p, _P, ctypes.c_size_t]
        L.bso_bs_map.restype = ctypes.c_double
        L.bso_bs_map.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_size_t] + [_P] * 7
        _lib = L
    return _lib


def ref_lib():
    """The compiled reference (None where its source tree was absent)."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        R = ctypes.CDLL(REF_SO)
        R.bsref_price_soa.restype = None
        R.bsref_price_soa.argtypes = [ctypes.c_size_t] + [_P] * 7
        R.bsref_cndf.restype = None
        R.bsref_cndf.argtypes = [ctypes.c_size_t, _P, _P]
        _ref = R
    return _ref


def _arrs(book):
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in book.arrays()[:5]]
    arrs.append(np.ascontiguousarray(book.otype, dtype=np.int32))
    return arrs


def _p(a):
    return a.ctypes.data_as(_P)


def price_ref(book) -> np.ndarray:
    """FP32 restatement (bit-identical to the reference)."""
    a = _arrs(book)
    out = np.empty(len(book), dtype=np.float32)
    lib().bso_price_ref_soa(len(book), *[_p(x) for x in a], _p(out))
    return out


def price_ref_cr(book) -> np.ndarray:
    """The FP32 restatement with exp/log correctly rounded to float in place
    of glibc's expf/logf: the rounding the reference-order GPU mode targets."""
    a = _arrs(book)
    out = np.empty(len(book), dtype=np.float32)
    lib().bso_price_ref_cr_soa(len(book), *[_p(x) for x in a], _p(out))
    return out


def price_fp64(book) -> np.ndarray:
    """FP64 evaluation of the same formula on the float32 inputs."""
    a = _arrs(book)
    out = np.empty(len(book), dtype=np.float64)
    lib().bso_price_fp64_soa(len(book), *[_p(x) for x in a], _p(out))
    return out


def d1_fp64(book) -> np.ndarray:
    s, k, r, v, t = (np.asarray(x, dtype=np.float64) for x in book.arrays()[:5])
    return ((r + v * v * 0.5) * t + np.log(s / k)) / (v * np.sqrt(t))


def price_reference(book):
    """The compiled reference's own BlkSchlsEqEuroNoDiv (None if not built)."""
    R = ref_lib()
    if R is None:
        return None
    a = _arrs(book)
    out = np.empty(len(book), dtype=np.float32)
    R.bsref_price_soa(len(book), *[_p(x) for x in a], _p(out))
    return out


def widened(book):
    """The book's five float arrays widened to double (NCO = 2 storage)."""
    return [np.ascontiguousarray(a, dtype=np.float64) for a in book.arrays()[:5]]


def price_fp64_d(s, k, r, v, t, otype) -> np.ndarray:
    """FP64 formula over double inputs."""
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (s, k, r, v, t)]
    ot = np.ascontiguousarray(otype, dtype=np.int32)
    out = np.empty(len(ot), dtype=np.float64)
    lib().bso_price_fp64_soa_d(len(ot), *[_p(x) for x in a], _p(ot), _p(out))
    return out


_simd = {}


def price_reference_simd(book, nco: int):
    """The reference's SIMD variant (blackscholes.simd.c:221-298) in packets of
    nco: 4 = SSE float on the float inputs, 2 = SSE2 double on the inputs
    widened to double.  None where it was not built (non-x86 machines)."""
    if nco not in _simd:
        path = REF_SIMD_SO[nco]
        if not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        fn = getattr(L, f"bsref_simd{nco}_price")
        fn.restype = None
        fn.argtypes = [ctypes.c_size_t] + [_P] * 7
        _simd[nco] = fn
    fn = _simd[nco]
    ot = np.ascontiguousarray(book.otype, dtype=np.int32)
    if nco == 4:
        a = _arrs(book)[:5]
        out = np.empty(len(book), dtype=np.float32)
    else:
        a = widened(book)
        out = np.empty(len(book), dtype=np.float64)
    fn(len(book), *[_p(x) for x in a], _p(ot), _p(out))
    return out


def cndf_ref(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    return np.array([lib().bso_cndf_ref(float(v)) for v in x], dtype=np.float32)


def static_partition(n: int, nw: int):
    b = np.empty(nw, dtype=np.int64)
    e = np.empty(nw, dtype=np.int64)
    lib().bso_static_partition(n, nw, _p(b), _p(e))
    return b, e


def read_parsec_fscanf(path, cap: int):
    """The reference's sequential parse; returns (Book, dgrefval)."""
    from p3arsec_gb300.books import Book
    a = [np.empty(cap, np.float32) for _ in range(5)]
    ot = np.empty(cap, np.int32)
    dg = np.empty(cap, np.float32)
    n = lib().bso_read_parsec_fscanf(os.fsencode(str(path)), cap, *[_p(x) for x in a], _p(ot), _p(dg))
    if n < 0:
        raise RuntimeError(f"cannot read {path}")
    return Book(*(x[:n] for x in a), ot[:n]), dg[:n]


def write_prices_fprintf(path, prices):
    p = np.ascontiguousarray(prices, dtype=np.float32)
    if lib().bso_write_prices_fprintf(os.fsencode(str(path)), _p(p), len(p)) != 0:
        raise RuntimeError(f"cannot write {path}")


_parsec = None


def _parsec_lib() -> ctypes.CDLL:
    """libbsoracle_parsec.so: bs_oracle.c built with PARSEC's flags."""
    global _parsec
    if _parsec is None:
        so = os.path.join(HERE, "libbsoracle_parsec.so")
        if not os.path.exists(so) or os.path.getmtime(so) < max(
                os.path.getmtime(os.path.join(HERE, f)) for f in ("bs_oracle.c", "swpt_oracle.c")):
            build(ref=False)
        L = ctypes.CDLL(so)
        L.bso_bs_map.restype = ctypes.c_double
        L.bso_bs_map.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_size_t] + [_P] * 7
        L.swo_price_all.restype = ctypes.c_double
        L.swo_price_all.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64,
                                    ctypes.c_int, _P, _P]
        _parsec = L
    return _parsec


def bs_map(book, nthreads: int, num_runs: int, parsec_flags: bool = False):
    """The threaded NUM_RUNS map driver; returns (prices, roi_seconds).
    parsec_flags: the build with PARSEC's compiler flags (-O3 -funroll-loops
    -fprefetch-loop-arrays, default contraction), as the reference is built
    -- the timed CPU baseline; its prices may differ from the checker's by
    fused multiply-adds on aarch64."""
    a = _arrs(book)
    out = np.empty(len(book), dtype=np.float32)
    L = _parsec_lib() if parsec_flags else lib()
    secs = L.bso_bs_map(nthreads, num_runs, len(book), *[_p(x) for x in a], _p(out))
    if secs < 0:
        raise RuntimeError("bso_bs_map failed")
    return out, secs


# ---------------------------------------------------------------- swaptions
class SwoSwaption(ctypes.Structure):
    """swo_swaption (swpt_oracle.h)."""
    _fields_ = [("strike", ctypes.c_double), ("compounding", ctypes.c_double),
                ("maturity", ctypes.c_double), ("tenor", ctypes.c_double),
                ("payment_interval", ctypes.c_double), ("years", ctypes.c_double),
                ("n_steps", ctypes.c_int), ("n_factors", ctypes.c_int),
                ("yield_", _P), ("factors", _P), ("seed", ctypes.c_uint64)]


def _swo_lib():
    L = lib()
    if not getattr(L, "_swo_ready", False):
        L.swo_price.restype = ctypes.c_int
        L.swo_price.argtypes = [ctypes.POINTER(SwoSwaption), ctypes.c_uint64, ctypes.c_uint,
                                ctypes.POINTER(ctypes.c_double)]
        L.swo_price_all.restype = ctypes.c_double
        L.swo_price_all.argtypes = [ctypes.POINTER(SwoSwaption), ctypes.c_int, ctypes.c_uint64,
                                    ctypes.c_int, _P, _P]
        L.swo_normal_pair.restype = None
        L.swo_normal_pair.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.POINTER(ctypes.c_double)]
        L.swo_yield_to_forward.restype = None
        L.swo_yield_to_forward.argtypes = [ctypes.c_int, _P, _P]
        L.swo_drift.restype = None
        L.swo_drift.argtypes = [ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, _P]
        L._swo_ready = True
    return L


def _swo_structs(swaptions):
    keep, arr = [], (SwoSwaption * max(len(swaptions), 1))()
    for i, s in enumerate(swaptions):
        y = np.ascontiguousarray(s.yield_curve, dtype=np.float64)
        f = np.ascontiguousarray(s.factors, dtype=np.float64)
        keep += [y, f]
        arr[i] = SwoSwaption(s.strike, s.compounding, s.maturity, s.tenor, s.payment_interval,
                             s.years, s.n_steps, s.n_factors, _p(y), _p(f), s.seed)
    return arr, keep


def swaption_price(swaption, trials: int, unfloored: bool = False):
    """(mean, standard error) of one swaption over `trials` paths; the whole
    HJM path matrix is simulated, as the reference does."""
    arr, keep = _swo_structs([swaption])
    out = (ctypes.c_double * 2)()
    if _swo_lib().swo_price(arr, trials, 1 if unfloored else 0, out) != 1:
        raise ValueError("swaption parameters out of the reference's range")
    return out[0], out[1]


def swaptions_all(swaptions, trials: int, nthreads: int, parsec_flags: bool = False):
    """Every swaption on nthreads threads (static partition, as the reference's
    ParallelFor); returns (prices, standard errors, wall seconds).
    parsec_flags: the build with PARSEC's compiler flags (the timed baseline)."""
    arr, keep = _swo_structs(swaptions)
    n = len(swaptions)
    price = np.empty(n)
    err = np.empty(n)
    L = _parsec_lib() if parsec_flags else _swo_lib()
    secs = L.swo_price_all(ctypes.cast(arr, ctypes.c_void_p) if parsec_flags else arr, n, trials,
                           nthreads, _p(price), _p(err))
    if secs < 0:
        raise ValueError("swaption parameters out of the reference's range")
    return price, err, secs


def normal_pair(seed: int, trial: int, j: int):
    z = (ctypes.c_double * 2)()
    _swo_lib().swo_normal_pair(seed, trial, j, z)
    return z[0], z[1]


def yield_to_forward(y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    f = np.empty_like(y)
    _swo_lib().swo_yield_to_forward(len(y), _p(y), _p(f))
    return f


def hjm_drift(factors, h: float):
    v = np.ascontiguousarray(factors, dtype=np.float64)
    mu = np.empty(v.shape[1])
    _swo_lib().swo_drift(v.shape[1] + 1, v.shape[0], _p(v), h, _p(mu))
    return mu
