"""The drop-in CLIs' argument handling, which runs before any GPU call:
the reference's usage message and exit(1) on bad options
(HJM_Securities.cpp:169-195)."""
import subprocess

from p3arsec_gb300 import build


def run(*args):
    build.build()
    return subprocess.run([build.SWAPTIONS_CLI, *args], stdout=subprocess.PIPE,
                          stderr=subprocess.PIPE, text=True, timeout=60)


def test_no_arguments_prints_usage_and_exits_1():
    r = run()
    assert r.returncode == 1 and "Usage:" in r.stderr and "PARSEC Benchmark Suite" in r.stdout


def test_unknown_option_exits_1():
    r = run("-xx", "3")
    assert r.returncode == 1 and "Unknown option: -xx" in r.stderr


def test_fewer_swaptions_than_threads_exits_1():
    r = run("-ns", "2", "-nt", "4")
    assert r.returncode == 1 and "Fewer swaptions than threads" in r.stderr
