"""bench.py's JSON contract, checked on the CPU through the reference arm
(the oracle port of the reference's FastFlow map on the host cores): one
JSON line with the contract's keys, at world size 1 and under torchrun at
world size 2 (rank 0 alone prints; the other rank exits 0 without work)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--options", "50000", "--steps", "2", "--warmup", "3", "--runs", "2"]
KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
        "cpu_baseline", "e2e"}


def json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def check_line(d):
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    assert d["config"]["workload"] and d["config"]["options"] == 50000
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_single_process():
    r = subprocess.run([sys.executable, "bench.py"] + ARGS, cwd=ROOT, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    check_line(lines[0])


def test_reference_arm_under_torchrun_two_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                        "--master-port", str(port), "bench.py", "--gpus", "2"] + ARGS,
                       cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1  # rank 0 only
    check_line(lines[0])


def test_both_arms_print_the_same_config():
    """The reference arm's config is the map's own config dict (no keys that
    only the GPU arm knows), so a comparison of the two lines' configs holds."""
    import bench
    r = subprocess.run([sys.executable, "bench.py"] + ARGS, cwd=ROOT, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json_lines(r.stdout)[0]
    assert line["config"] == bench.map_config(50000, 2, 1)
    assert line["cpu_baseline"]["note"]


def test_prefix_bytes_follows_the_library_rule():
    import bench
    l2 = 135528448.0
    tune = {"load_path": 7, "resident_32nds": 10}
    # 10/32 of the L2 in whole 8-option groups of 28 bytes
    assert bench.prefix_bytes(tune, 10_000_000, l2) == (int(l2) * 10 // 32 // 224) * 224
    assert bench.prefix_bytes({"load_path": 7, "resident_32nds": 0}, 10_000_000, l2) == \
        (int(l2) * 15 // 32 // 224) * 224
    assert bench.prefix_bytes({"load_path": 2}, 10_000_000, l2) == 0
    assert bench.prefix_bytes(tune, 1000, l2) == 1000 // 8 * 8 * 28  # the whole (small) book



def _pt(rate, p99, ops, done=True):
    return {"rate_per_s": rate, "median_p99_ms": p99, "median_options_per_s": ops,
            "all_completed": done}


def test_equal_p99_picks_the_best_rate_within_each_bound():
    import bench
    sweep = {"batched": [_pt(50e3, 0.4, 5e9), _pt(60e3, 0.9, 6e9), _pt(70e3, 1.6, 7e9),
                         _pt(80e3, 1.9, 7.5e9, done=False)],   # a trace that did not drain
             "plain": [_pt(1e3, 0.7, 1e8), _pt(5e3, 0.95, 5e8), _pt(10e3, 3.0, 9e8)]}
    eq = {e["p99_bound_ms"]: e for e in bench.equal_p99(sweep, (0.5, 1.0, 2.0), 8.8e9)}
    # 1 ms: batched 60k (6e9), plain 5k (5e8)
    assert eq[1.0]["batched_rate_per_s"] == 60e3 and eq[1.0]["plain_rate_per_s"] == 5e3
    assert eq[1.0]["ratio"] == 6e9 / 5e8 and eq[1.0]["ratio_ceiling_from_link"] == 8.8e9 / 5e8
    # 2 ms: the undrained 80k point does not count
    assert eq[2.0]["batched_rate_per_s"] == 70e3 and eq[2.0]["ratio"] == 7e9 / 5e8
    # 0.5 ms: the plain loop meets it at no rate -- null ratio and a note
    assert eq[0.5]["ratio"] is None and eq[0.5]["ratio_ceiling_from_link"] is None
    assert "every swept rate" in eq[0.5]["plain_note"] and "0.70 ms" in eq[0.5]["plain_note"]
    assert "batched_note" not in eq[0.5]
