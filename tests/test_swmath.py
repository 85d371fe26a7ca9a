"""The swaption Monte Carlo's elementary functions (p3arsec_gb300/csrc/bsg_swmath.h):
the normal variates (Box-Muller with table-driven -2 ln u and sin/cos(2 pi u)
computed from the uniforms' bits) and the discount factors' exp.  On the
CPU, the host build of the same header against long-double
logl/sinl/cosl/expl; on the GPU, the device transform against the host
build, bit for bit, and against a long-double evaluation of the textbook
formula."""
import os
import re
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "p3arsec_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("swmath") / "swmath_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "swmath_check.cpp"), "-o", exe], check=True)
    return exe


def test_accuracy_against_long_double(checker):
    """2M random uniforms plus u next to 0 and 1 and every table boundary:
    -2 ln u within 2 ulp, sin and cos within 1.2e-16, the normals within
    5.2e-16 of max(1, |z|); 2.5M arguments of exp, its reduction's grid
    points and rounding boundaries among them: within 1.1 ulp."""
    r = subprocess.run([checker, "walk", "2000000", "1"], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    m = re.search(r"checked (\d+) log_ulp (\S+) trig_abs (\S+) z_rel (\S+) exp_ulp (\S+)", r.stdout)
    checked, log_ulp, trig, zrel, exp_ulp = int(m.group(1)), *(float(g) for g in m.groups()[1:])
    assert checked > 4_500_000
    assert log_ulp <= 2.0 and trig <= 1.2e-16 and zrel <= 5.2e-16, r.stdout
    assert exp_ulp <= 1.1, r.stdout


def test_table_header_is_what_the_generator_writes(tmp_path):
    """bsg_swmath_tables.h is generated: regenerating it changes nothing."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen", os.path.join(CSRC, "gen_swmath_tables.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    gen.HERE = str(tmp_path)
    gen.main()
    with open(os.path.join(CSRC, "bsg_swmath_tables.h")) as a, \
            open(tmp_path / "bsg_swmath_tables.h") as b:
        assert a.read() == b.read()


def _words(n, seed):
    """n random word quadruples plus quadruples of edge uniforms (u next to
    0 and 1, the 1/128 and 1/256 grid points and midpoints)."""
    rng = np.random.default_rng(seed)
    w = rng.integers(0, 1 << 32, size=(n, 4), dtype=np.uint64).astype(np.uint32)
    kmax = (1 << 52) - 1
    ks = [0, 1, 2, kmax, kmax - 1, 1 << 51, (1 << 51) - 1, 3 << 50]
    ks += [(j << sh) + e + d for j in range(257) for sh in (44, 45) for e in (0, 1 << 43)
           for d in (-1, 0, 1) if 0 <= (j << sh) + e + d <= kmax]
    edge = []
    for i, k in enumerate(ks):
        k2 = ks[(7 * i + 3) % len(ks)]
        edge.append([(k >> 32) << 12, k & 0xFFFFFFFF, (k2 >> 32) << 12, k2 & 0xFFFFFFFF])
    return np.concatenate([w, np.array(edge, dtype=np.uint64).astype(np.uint32)])


def _textbook(words):
    """z0, z1 from long-double log, sqrt, cos and sin of the same uniforms
    (numpy's longdouble: 64-bit mantissa on x86, 113-bit on Arm)."""
    L = np.longdouble
    w = words.astype(np.uint64)
    k1 = ((w[:, 0] >> np.uint64(12)) << np.uint64(32)) | w[:, 1]
    k2 = ((w[:, 2] >> np.uint64(12)) << np.uint64(32)) | w[:, 3]
    u1 = (2 * k1 + 1).astype(L) / L(2) ** 53
    u2 = (2 * k2 + 1).astype(L) / L(2) ** 53
    r = np.sqrt(-2 * np.log(u1))
    th = 2 * L("3.141592653589793238462643383279502884") * u2
    return np.stack([r * np.cos(th), r * np.sin(th)], axis=1).ravel()


@pytest.mark.gpu
def test_device_transform_equals_the_host_build(gpu_ctx, checker, tmp_path):
    words = _words(1 << 20, seed=5)
    z = gpu_ctx.swaption_normals(words)
    inp, out = tmp_path / "w.bin", tmp_path / "z.bin"
    words.tofile(inp)
    subprocess.run([checker, "pairs", str(inp), str(out)], check=True, timeout=120)
    host = np.fromfile(out, dtype=np.float64)
    assert host.size == z.size == 2 * len(words)
    assert np.array_equal(z.view(np.uint64), host.view(np.uint64))
    # and the textbook formula in long double
    ref = _textbook(words)
    err = np.abs(z.astype(np.longdouble) - ref) / np.maximum(1, np.abs(ref))
    assert float(err.max()) <= 6e-16
    # the transform is a normal sampler: moments of the 2M variates
    zr = z[: 2 << 20]
    assert abs(zr.mean()) < 5e-3 and abs(zr.std() - 1) < 5e-3


@pytest.mark.gpu
def test_device_transform_refuses_bad_arguments(gpu_ctx):
    with pytest.raises(ValueError):
        gpu_ctx.swaption_normals(np.zeros(6, dtype=np.uint32))
    assert gpu_ctx.lib.bsg_swaption_normals(gpu_ctx.h, 0, 4, 0) == -1  # BSG_ERR_INVALID_ARG
