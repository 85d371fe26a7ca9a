"""The persistent serving kernel's tile-claim protocol (csrc/bsg_ring.h),
run on the CPU by threads through the same header the kernel compiles: a
host thread publishing requests into a small ring that is reused hundreds
of times, worker threads claiming and completing tiles with stale views of
the current request.  Every tile must be claimed exactly once and every
request completed exactly once, after all its tiles."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "p3arsec_gb300", "csrc")


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("ring") / "ring_model_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC,
                    os.path.join(HERE, "ring_model_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("requests,workers,ring,seed", [
    (20000, 8, 8, 1),     # every slot reused ~2500 times
    (20000, 3, 4, 2),
    (5000, 16, 2, 3),     # two slots, many more workers than requests in flight
    (30000, 6, 64, 4),
])
def test_claim_protocol_exactly_once(model, requests, workers, ring, seed):
    r = subprocess.run([model, str(requests), str(workers), str(ring), str(seed)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert r.stdout.startswith("ok"), r.stdout


@pytest.mark.parametrize("seed", range(10, 30))
def test_claim_protocol_two_slots_many_workers(model, seed):
    """Two slots and sixteen workers: slots are re-armed while stale workers
    still add to them, the case where a blind add takes a later request's
    tile (which the worker must then price)."""
    r = subprocess.run([model, "600", "16", "2", str(seed)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout


@pytest.mark.parametrize("requests,workers,ring,seed,window", [
    (10000, 8, 8, 1, 8),    # the window as wide as the ring
    (10000, 16, 4, 2, 2),
    (3000, 16, 2, 3, 2),    # two slots: re-armed words under windowed claims
    (20000, 12, 64, 4, 32),
    (20000, 6, 4096, 5, 32),  # the kernel's ring and window
])
def test_windowed_claims_exactly_once(model, requests, workers, ring, seed, window):
    """Workers spread over the oldest `window` published requests
    (claim_window, starting at rotating offsets; the oldest advanced past
    once exhausted): still every tile claimed exactly once and every request
    completed once."""
    r = subprocess.run([model, str(requests), str(workers), str(ring), str(seed), str(window)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
