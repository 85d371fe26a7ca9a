"""The serving loop: continuous batching, admission by memory budget, and
host-side failure handling (cancel, bounded waits).  No test faults or hangs
the GPU: failures are made on the host (a paused loop, a cancelled request,
an oversized request)."""
import threading

import numpy as np
import pytest

from p3arsec_gb300 import books
from p3arsec_gb300.abi import BsgError, Server, serve_trace

pytestmark = pytest.mark.gpu

OK, TIMEOUT, CANCELLED, BUDGET, CAPACITY, STATE = 0, -7, -9, -8, -5, -11
KINDS = {"unfused": dict(fused=False), "fused": dict(fused=True),
         "persistent": dict(persistent=True),
         # the persistent kernel's blocks shared by the 16 oldest requests
         "persistent_w16": dict(persistent=True, persistent_window=16)}


def pinned_book(torch, n, seed):
    book = books.generate(n, seed=seed)
    arrs = [torch.from_numpy(a).pin_memory().numpy() for a in book.arrays()]
    return book, arrs


def pinned_zeros(torch, n):
    return torch.zeros(n, dtype=torch.float32).pin_memory().numpy()


def disjoint_requests(rng, pool_n, count, max_n):
    """(offset, n) of `count` non-overlapping requests inside the pool."""
    cuts = np.sort(rng.choice(pool_n, size=2 * count, replace=False))
    reqs = []
    for i in range(count):
        a, b = int(cuts[2 * i]), int(cuts[2 * i + 1])
        reqs.append((a, max(1, min(b - a, max_n))))
    return reqs


@pytest.mark.parametrize("kind", list(KINDS))
def test_each_result_same_alone_and_in_mix(gpu_ctx, kind):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    pool_n = 1 << 21
    book, host = pinned_book(torch, pool_n, 41)
    mix = pinned_zeros(torch, pool_n)
    alone = pinned_zeros(torch, pool_n)
    reqs = disjoint_requests(rng, pool_n, 400, 40000)
    with Server(budget_bytes=256 << 20, max_inflight=4, **KINDS[kind]) as srv:
        for a in host + [mix, alone]:
            srv.register(a)
        # the mix: four threads submit concurrently while admission is held,
        # so the loop coalesces them into shared batches when it resumes
        ids = [None] * len(reqs)

        def client(part):
            for i in part:
                o, n = reqs[i]
                ids[i] = srv.submit(*[a[o:] for a in host], mix[o:], n=n)

        srv.pause(True)
        th = [threading.Thread(target=client, args=(range(j, len(reqs), 4),)) for j in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        srv.pause(False)
        for rid in ids:
            st, lat = srv.wait(rid, timeout_s=60.0)
            assert st == OK and lat > 0
        stats = srv.stats()
        assert stats["completed"] == len(reqs)
        if kind.startswith("persistent"):
            # every request went to the one running kernel (relaunched at
            # most after an idle exit), none needed a launch of its own
            assert stats["kernel_launches"] <= 3
        else:
            assert stats["batches"] < len(reqs) / 4  # requests were coalesced
            # batches of more than 24 requests take the copied-table launch,
            # the single requests below the table-in-parameters launch
            assert stats["max_batch_requests_seen"] > 24
        # alone: one request in flight at a time
        for o, n in reqs[:50]:
            st, _ = srv.wait(srv.submit(*[a[o:] for a in host], alone[o:], n=n), timeout_s=60.0)
            assert st == OK
    ref = gpu_ctx.price_book(book)
    for i, (o, n) in enumerate(reqs):
        assert np.array_equal(mix[o:o + n].view(np.uint32), ref[o:o + n].view(np.uint32)), i
    for o, n in reqs[:50]:
        assert np.array_equal(alone[o:o + n].view(np.uint32), mix[o:o + n].view(np.uint32))


@pytest.mark.parametrize("mode", ["sfu_ref", "libm_ref"])
@pytest.mark.parametrize("kind", list(KINDS))
def test_reference_order_modes_serve_the_maps_bits(gpu_ctx, kind, mode):
    """The serving kernels in the reference-order modes: a mix of requests
    (heads and tails off the vector grid, one option to 3 tiles) priced as
    the map prices the same options in the same mode, bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    pool_n = 1 << 18
    book, host = pinned_book(torch, pool_n, 43)
    out = pinned_zeros(torch, pool_n)
    reqs = disjoint_requests(rng, pool_n, 60, 6000)
    with Server(budget_bytes=64 << 20, max_inflight=4, mode=mode, **KINDS[kind]) as srv:
        for a in host + [out]:
            srv.register(a)
        ids = [srv.submit(*[a[o:] for a in host], out[o:], n=n) for o, n in reqs]
        for rid in ids:
            st, _ = srv.wait(rid, timeout_s=60.0)
            assert st == OK
    ref = gpu_ctx.price_book(book, mode=mode)
    for i, (o, n) in enumerate(reqs):
        assert np.array_equal(out[o:o + n].view(np.uint32), ref[o:o + n].view(np.uint32)), i


@pytest.mark.parametrize("kind", list(KINDS))
def test_empty_requests_complete_at_once_among_others(gpu_ctx, kind):
    torch = pytest.importorskip("torch")
    book, host = pinned_book(torch, 1 << 16, 47)
    out = pinned_zeros(torch, 1 << 16)
    with Server(budget_bytes=64 << 20, max_inflight=4, **KINDS[kind]) as srv:
        for a in host + [out]:
            srv.register(a)
        ids = []
        for i, (o, n) in enumerate([(0, 0), (100, 5000), (9000, 0), (20000, 3), (30000, 0)]):
            ids.append((o, n, srv.submit(*[a[o:] for a in host], out[o:], n=n)))
        for o, n, rid in ids:
            st, _ = srv.wait(rid, timeout_s=60.0)
            assert st == OK, (o, n)
        assert srv.stats()["completed"] == 5
    ref = gpu_ctx.price_book(book)
    for o, n, _ in ids:
        assert np.array_equal(out[o:o + n].view(np.uint32), ref[o:o + n].view(np.uint32))
    assert out[9000] == 0.0 and out[30000] == 0.0  # the empty requests wrote nothing


def test_plain_mode_same_bits(gpu_ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    pool_n = 1 << 19
    book, host = pinned_book(torch, pool_n, 42)
    out = pinned_zeros(torch, pool_n)
    reqs = disjoint_requests(rng, pool_n, 60, 20000)
    with Server(budget_bytes=64 << 20, plain=True) as srv:
        ids = [srv.submit(*[a[o:] for a in host], out[o:], n=n) for o, n in reqs]
        for rid in ids:
            assert srv.wait(rid, timeout_s=60.0)[0] == OK
        assert srv.stats()["batches"] == len(reqs)
    ref = gpu_ctx.price_book(book)
    for o, n in reqs:
        assert np.array_equal(out[o:o + n].view(np.uint32), ref[o:o + n].view(np.uint32))


def test_cancel_and_bounded_wait():
    torch = pytest.importorskip("torch")
    _, host = pinned_book(torch, 100000, 43)
    out = pinned_zeros(torch, 100000)
    with Server(budget_bytes=64 << 20) as srv:
        for a in host + [out]:
            srv.register(a)
        srv.pause(True)
        held = srv.submit(*host, out, n=1000)
        other = srv.submit(*host, out, n=2000)
        st, _ = srv.wait(held, timeout_s=0.05)
        assert st == TIMEOUT  # still queued, still pending
        assert srv.cancel(held) == OK
        assert srv.wait(held, timeout_s=1.0)[0] == CANCELLED
        assert srv.stats()["queued"] == 1
        srv.pause(False)
        assert srv.wait(other, timeout_s=60.0)[0] == OK
        assert srv.cancel(srv.submit(*host, out, n=10)) in (OK, STATE)


@pytest.mark.parametrize("kind", ["fused", "persistent"])
def test_admission_by_budget(gpu_ctx, kind):
    torch = pytest.importorskip("torch")
    pool_n = 600000
    book, host = pinned_book(torch, pool_n, 44)
    out = pinned_zeros(torch, pool_n)
    budget = 28 * 131072  # room for one 100k request at a time
    with Server(budget_bytes=budget, max_inflight=4, **KINDS[kind]) as srv:
        for a in host + [out]:
            srv.register(a)
        with pytest.raises(BsgError) as e:
            srv.submit(*host, out, n=200000)
        assert e.value.status == BUDGET
        ids = [srv.submit(*[a[o:] for a in host], out[o:], n=100000)
               for o in range(0, 500000, 100000)]
        for rid in ids:
            assert srv.wait(rid, timeout_s=60.0)[0] == OK
        if kind == "fused":
            assert srv.stats()["max_batch_requests_seen"] == 1
    ref = gpu_ctx.price_book(book)
    assert np.array_equal(out[:500000].view(np.uint32), ref[:500000].view(np.uint32))


def test_unregistered_host_memory_is_rejected():
    torch = pytest.importorskip("torch")
    book = books.generate(1000, seed=45)
    out = np.zeros(1000, dtype=np.float32)
    with Server(budget_bytes=64 << 20) as srv:
        with pytest.raises(BsgError):
            srv.submit(*book.arrays(), out)
        # registering a range larger than an existing pinned block is refused
        pinned = torch.zeros(1000, dtype=torch.float32).pin_memory()
        assert srv.lib.bsg_server_register(srv.h, pinned.data_ptr(), 1 << 30) != 0


@pytest.mark.parametrize("plain,kind", [(False, "unfused"), (False, "fused"),
                                        (False, "persistent"), (True, "unfused")])
def test_short_trace(plain, kind):
    torch = pytest.importorskip("torch")
    pool_n = 1 << 20
    _, host = pinned_book(torch, pool_n, 46)
    out = pinned_zeros(torch, pool_n)
    lat = np.zeros(5000)
    res = serve_trace(host, out, rate_per_s=1000, duration_s=0.5, min_n=16, max_n=1 << 16,
                      seed=3, budget_bytes=1 << 30, plain=plain, latencies=lat, **KINDS[kind])
    assert res["requests"] > 300
    assert res["completed"] == res["requests"]
    assert 0 < res["p50_s"] <= res["p99_s"] <= res["max_s"] < 10
    assert np.isfinite(lat[:res["requests"]]).all()


def test_persistent_kernel_exits_when_idle_and_relaunches(gpu_ctx):
    """The persistent kernel's only wait (for published work) is bounded:
    with nothing published for longer than its 5 ms bound every block exits
    by itself (a host-side omission, no fault); the next request relaunches
    the kernel and completes."""
    import time
    torch = pytest.importorskip("torch")
    book, host = pinned_book(torch, 300000, 47)
    out = pinned_zeros(torch, 300000)
    with Server(budget_bytes=64 << 20, persistent=True) as srv:
        for a in host + [out]:
            srv.register(a)
        assert srv.wait(srv.submit(*host, out, n=100000), timeout_s=60.0)[0] == OK
        assert srv.stats()["kernel_launches"] == 1
        time.sleep(0.05)  # ten idle bounds: the kernel has exited
        assert srv.wait(srv.submit(*[a[100000:] for a in host], out[100000:], n=200000),
                        timeout_s=60.0)[0] == OK
        assert srv.stats()["kernel_launches"] == 2
    ref = gpu_ctx.price_book(book)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_persistent_request_size_limit():
    torch = pytest.importorskip("torch")
    _, host = pinned_book(torch, 1000, 48)
    out = pinned_zeros(torch, 1000)
    with Server(budget_bytes=1 << 30, persistent=True) as srv:
        for a in host + [out]:
            srv.register(a)
        # checked before any array is touched: 4095 tiles of 2048 options
        with pytest.raises(BsgError) as e:
            srv.submit(*host, out, n=4095 * 2048 + 1)
        assert e.value.status == CAPACITY
        assert srv.wait(srv.submit(*host, out, n=1000), timeout_s=60.0)[0] == OK
