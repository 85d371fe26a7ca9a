"""include/bsg_map.cuh: the generic elementwise map (the SkePU2 Map<N>
counterpart).  The CPU test compiles the harness for sm_103a; the GPU tests
run it against bsg_price_soa (bit for bit) and exact references."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from p3arsec_gb300 import books
from p3arsec_gb300 import build as b

SRC = os.path.join(ROOT, "tests", "map_skeleton_check.cu")


def _nvcc(out, extra):
    cmd = [b.nvcc()] + b.ARCH + ["-O3", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                                 "-I" + b.CSRC] + extra + [SRC, "-o", out]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


def test_skeleton_compiles_for_sm103a(tmp_path):
    _nvcc(str(tmp_path / "skel.o"), ["-c"])


@pytest.fixture(scope="module")
def skel(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("skel") / "libskel.so")
    _nvcc(so, ["-shared", "-Xcompiler", "-fPIC"])
    L = ctypes.CDLL(so)
    P = ctypes.c_void_p
    L.skel_bs.argtypes = [ctypes.c_int64] + [P] * 7 + [ctypes.c_int, ctypes.c_int]
    L.skel_axpy.argtypes = [ctypes.c_int64, ctypes.c_float, P, P, P]
    L.skel_mixed.argtypes = [ctypes.c_int64, P, P, P, P]
    return L


@pytest.mark.gpu
@pytest.mark.parametrize("n,pad", [(1, 0), (7, 0), (100003, 0), (4099, 1)])
def test_blackscholes_through_the_skeleton(gpu_ctx, skel, n, pad):
    torch = pytest.importorskip("torch")
    book = books.generate(n, seed=61)
    want = gpu_ctx.price_book(book)
    dev = []
    for a in book.arrays():
        t = torch.zeros(n + pad, dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                        device="cuda:0")
        t[pad:] = torch.from_numpy(a).cuda()
        dev.append(t[pad:])
    out = torch.zeros(n + pad, dtype=torch.float32, device="cuda:0")[pad:]
    for pdl in (0, 1):
        assert skel.skel_bs(n, *[x.data_ptr() for x in dev], out.data_ptr(), pdl, 3) == 0
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_axpy_and_mixed_types(skel):
    torch = pytest.importorskip("torch")
    n = 1000003
    rng = np.random.default_rng(3)
    x = rng.integers(-1000, 1000, n).astype(np.float32)
    y = rng.integers(-1000, 1000, n).astype(np.float32)
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    out = torch.empty(n, dtype=torch.float32, device="cuda:0")
    assert skel.skel_axpy(n, 3.0, dx.data_ptr(), dy.data_ptr(), out.data_ptr()) == 0
    assert np.array_equal(out.cpu().numpy(), 3.0 * x + y)
    i = rng.integers(-50, 50, n).astype(np.int32)
    f = rng.standard_normal(n).astype(np.float32)
    d = rng.standard_normal(n)
    di, df, dd = (torch.from_numpy(a).cuda() for a in (i, f, d))
    o = torch.empty(n, dtype=torch.float64, device="cuda:0")
    assert skel.skel_mixed(n, di.data_ptr(), df.data_ptr(), dd.data_ptr(), o.data_ptr()) == 0
    assert np.array_equal(o.cpu().numpy(), i.astype(np.float64) + f.astype(np.float64) * d)
