"""include/bsg_compat.h: a caller written against the reference's batch
signature (blackscholes.simd.c:221-223) compiles unchanged against the
header, links libbsgpu.so, and prices on the GPU with the library's bits --
in one call and in the reference's packets of NCO = 4 options
(blackscholes.simd.c:376-383)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "compat_caller.c")


def build_caller(tmp_path):
    from p3arsec_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "compat_caller")
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           SRC, "-o", exe, "-L" + os.path.dirname(lib), "-lbsgpu",
           "-Wl,-rpath," + os.path.dirname(lib), "-Wl,--no-undefined"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return exe


def test_reference_signature_compiles_and_links(tmp_path):
    build_caller(tmp_path)


@pytest.mark.gpu
def test_reference_signature_prices_like_the_library(tmp_path, gpu_ctx):
    from p3arsec_gb300 import books
    exe = build_caller(tmp_path)
    n = 4096
    book = books.generate(n, seed=31)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.int32(n).tobytes())
        for a in book.arrays():
            f.write(np.ascontiguousarray(a).tobytes())
    r = subprocess.run([exe, str(inp)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    bits = np.array([[int(x, 16) for x in line.split()] for line in r.stdout.split("\n") if line],
                    dtype=np.uint32)
    assert bits.shape == (n, 2)
    want = gpu_ctx.price_book(book, num_runs=1).view(np.uint32)
    assert np.array_equal(bits[:, 0], want)
    assert np.array_equal(bits[:, 1], want)
