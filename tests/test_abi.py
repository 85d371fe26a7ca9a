"""The C-ABI library: loads, exports every declared symbol (no GPU calls)."""
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "bsg.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(bsg_\w+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def lib():
    from p3arsec_gb300 import build
    build.build()
    from p3arsec_gb300 import abi
    return abi.load()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert "bsg_price_soa" in syms and "bsg_create" in syms
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_covers_the_header(lib):
    from p3arsec_gb300 import abi
    assert set(declared_symbols()) == set(abi.SIGNATURES)


def test_no_cpu_fallback_without_gpu(lib):
    from p3arsec_gb300 import abi
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(abi.BsgError) as e:
        abi.Context(0, 16)
    assert e.value.status == -2  # BSG_ERR_NO_DEVICE


def test_strerror(lib):
    assert lib.bsg_strerror(0) == b"ok"
    assert b"capacity" in lib.bsg_strerror(-5)


def test_library_does_not_link_the_oracle():
    so = os.path.join(ROOT, "p3arsec_gb300", "libbsgpu.so")
    data = open(so, "rb").read()
    assert b"libbsoracle" not in data and b"bso_price" not in data


def test_noalloc_refuses_reference_order_modes_before_any_cuda_call(lib):
    """bsg_price_batch_noalloc prices in the fast mode only; a mode flag is
    refused by the argument check, which runs before any CUDA call (so this
    holds on a machine without a GPU)."""
    from p3arsec_gb300 import abi
    seg = (abi.Segment * 1)()
    seg[0].offset, seg[0].len = 0, 1
    for mode in ("sfu_ref", "libm_ref"):
        st = lib.bsg_price_batch_noalloc(None, None, None, None, None, None, None, 1, seg, 1,
                                         None, abi.MODES[mode])
        assert st == -1  # BSG_ERR_INVALID_ARG
