"""Serving control logic on the CPU with a fake executor (no GPU)."""
import threading
import time

import numpy as np
import pytest

from slakonet_gb300 import serving as SV, synthetic as syn


class FakeModel:
    pass


def _structs(n, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        st = syn.random_structure(rng, int(rng.integers(1, 6)), zmax=20)
        st["kpoints"] = np.zeros((int(rng.integers(1, 5)), 3))
        out.append(st)
    return out


def test_admission_budget_never_exceeded_and_all_requests_complete():
    peak = {"v": 0}
    live = {"v": 0}
    lock = threading.Lock()

    def fake_exec(structures, stream):
        with lock:
            live["v"] += len(structures)
            peak["v"] = max(peak["v"], server.adm.used)
        time.sleep(0.01)
        with lock:
            live["v"] -= len(structures)
        return [{"eigenvalues": np.zeros(1), "band_gap_eV": 0.0} for _ in structures]

    sd = syn.default_shell_dict()
    sts = _structs(60)
    budget = 3 * SV.request_bytes(16, 4, 1000)
    server = SV.Server(FakeModel(), sd, device="cpu", mem_budget_bytes=budget, n_workers=3, executor=fake_exec)
    lat, wall, res = SV.poisson_stream(server, sts, rate=2000.0, seed=1)
    server.close()
    assert len(lat) == len(sts)
    assert peak["v"] <= budget
    assert server.adm.used == 0
    assert server.batches >= 2


def test_oversized_request_is_rejected_not_queued():
    sd = syn.default_shell_dict()
    st = {"numbers": np.array([60] * 600), "positions": np.zeros((600, 3)), "cell": np.eye(3) * 50,   # 9600 orbitals
          "kpoints": np.zeros((1, 3))}
    server = SV.Server(FakeModel(), sd, device="cpu", mem_budget_bytes=1 << 30, n_workers=1,
                       executor=lambda s, stream: [{} for _ in s])
    f = server.submit(st)
    server.close()
    assert f.exception() is not None and server.rejected == 1


def test_batches_form_from_requests_that_arrive_during_execution():
    sd = syn.default_shell_dict()
    sizes = []

    def slow_exec(structures, stream):
        sizes.append(len(structures))
        time.sleep(0.05)
        return [{} for _ in structures]

    server = SV.Server(FakeModel(), sd, device="cpu", mem_budget_bytes=1 << 40, n_workers=1, executor=slow_exec)
    sts = _structs(20, seed=3)
    futs = [server.submit(sts[0])]
    time.sleep(0.01)
    futs += [server.submit(s) for s in sts[1:]]
    for f in futs:
        f.result(timeout=10)
    server.close()
    # the first batch holds one request; the rest arrived while it ran and were batched together
    assert sizes[0] == 1 and max(sizes[1:]) > 1


def test_malformed_requests_are_refused_alone_and_batch_mates_complete():
    server, gate, seen = _gated_server()
    good = [server.submit(_atoms(2)), server.submit(_atoms(3))]
    bad = {"positions for": dict(_atoms(2), positions=np.zeros((3, 3))),
           "k-point weights": dict(_atoms(2), weights=np.ones(4)),
           "non-finite": dict(_atoms(2), cell=np.diag([10.0, np.nan, 10.0])),
           "no shells for element": dict(_atoms(2), numbers=np.array([1, 200]))}
    futs = {m: server.submit(st) for m, st in bad.items()}
    gate.set()
    for m, f in futs.items():
        with pytest.raises(ValueError, match=m):
            f.result(timeout=10)
    assert [f.result(timeout=10)["n"] for f in good] == [2, 3]
    server.close()
    assert server.rejected == len(bad) and all(n in (2, 3) for b in seen for n in b)
    assert server.adm.used == 0


def test_close_finishes_every_submitted_request_and_refuses_new_ones():
    def slow(structures, stream):
        time.sleep(0.01)
        return [{"n": len(s["numbers"])} for s in structures]

    # room for about two requests at a time, so most of them still wait for admission at close()
    budget = 2 * SV.request_bytes(4, 1, 1000) + 1
    server = SV.Server(FakeModel(), syn.default_shell_dict(), device="cpu", mem_budget_bytes=budget, n_workers=2,
                       executor=slow)
    futs = [server.submit(_atoms(1 + i % 3)) for i in range(29)]
    server.close()
    assert all(f.done() for f in futs)
    assert [f.result()["n"] for f in futs] == [1 + i % 3 for i in range(29)]
    late = server.submit(_atoms(2))
    with pytest.raises(RuntimeError, match="closed"):
        late.result(timeout=1)
    server.close()                                       # a second close is a no-op
    assert server.adm.used == 0


def _gated_server(fail_marker=None):
    """One worker whose executor waits for ``gate`` and fails any batch holding ``fail_marker`` atoms."""
    gate = threading.Event()
    seen = []

    def execute(structures, stream):
        gate.wait(10)
        seen.append([len(s["numbers"]) for s in structures])
        if fail_marker is not None and any(len(s["numbers"]) == fail_marker for s in structures):
            raise RuntimeError("simulated executor failure")
        return [{"n": len(s["numbers"])} for s in structures]

    server = SV.Server(FakeModel(), syn.default_shell_dict(), device="cpu", mem_budget_bytes=1 << 40,
                       n_workers=1, executor=execute)
    return server, gate, seen


def _atoms(n):
    return {"numbers": np.ones(n, dtype=np.int64), "positions": np.zeros((n, 3)), "cell": np.eye(3) * 10,
            "kpoints": np.zeros((1, 3))}


def _wait_for(pred, timeout=10.0):
    t = time.time()
    while not pred() and time.time() - t < timeout:
        time.sleep(0.005)
    assert pred()


def test_executor_failure_reaches_every_request_of_its_batch_and_serving_continues():
    server, gate, seen = _gated_server(fail_marker=7)
    first = server.submit(_atoms(1))                    # occupies the worker until the gate opens
    _wait_for(lambda: server.adm.used > 0 and not server.ready)
    mix = [server.submit(_atoms(n)) for n in (2, 7, 3)]  # queued together behind it; 7 atoms fails the batch
    _wait_for(lambda: len(server.ready) == 3)
    gate.set()
    assert first.result(timeout=10) == {"n": 1, "latency_s": first.result()["latency_s"]}
    for f in mix:
        with pytest.raises(RuntimeError, match="simulated executor failure"):
            f.result(timeout=10)
    after = server.submit(_atoms(4))
    assert after.result(timeout=10)["n"] == 4             # the worker survived the failed batch
    server.close()
    assert seen == [[1], [2, 3, 7], [4]]                 # the batch runs cheapest first
    assert server.adm.used == 0                          # every request's memory was released


def test_cancelled_request_is_dropped_before_execution_and_worker_survives():
    server, gate, seen = _gated_server()
    first = server.submit(_atoms(1))
    _wait_for(lambda: server.adm.used > 0 and not server.ready)
    cancelled, kept = server.submit(_atoms(5)), server.submit(_atoms(6))
    _wait_for(lambda: len(server.ready) == 2)
    assert cancelled.cancel()
    gate.set()
    assert first.result(timeout=10)["n"] == 1 and kept.result(timeout=10)["n"] == 6
    assert cancelled.cancelled()
    after = server.submit(_atoms(2))
    assert after.result(timeout=10)["n"] == 2
    server.close()
    assert [5] not in seen and all(5 not in b for b in seen)
    assert server.adm.used == 0


_KEYS = ("numbers", "positions", "cell", "kpoints", "weights")


def _same(a, b):
    return len(a) == len(b) and all(np.array_equal(x[k], y[k]) for x, y in zip(a, b) for k in _KEYS)


def test_serving_request_set_is_chunked_seeded_and_independent_of_processes():
    serial = syn.serving_requests(5, chunk=2)
    parallel = syn.serving_requests(5, chunk=2, processes=2)
    assert _same(serial, parallel)
    # chunk i is uneven_batch(seed = 1000 + i); one seeded permutation interleaves the chunks
    chunks = (syn.uneven_batch(2, nmin=1, nmax=200, zmax=65, seed=1000)
              + syn.uneven_batch(2, nmin=1, nmax=200, zmax=65, seed=1001)
              + syn.uneven_batch(1, nmin=1, nmax=200, zmax=65, seed=1002))
    order = np.random.default_rng(5).permutation(5)
    for st, i in zip(serial, order):
        for k in ("numbers", "positions", "cell", "kpoints"):
            assert np.array_equal(st[k], chunks[i][k])
        assert np.allclose(st["weights"].sum(), 1.0) and len(st["weights"]) == len(st["kpoints"])
        assert 1 <= len(st["numbers"]) <= 200


def test_serving_request_file_round_trip_and_bench_loader(tmp_path):
    import importlib.util
    import os
    sts = syn.serving_requests(3, chunk=625)
    path = str(tmp_path / "requests.npz")
    syn.save_structures(path, sts)
    assert _same(sts, syn.load_structures(path))
    spec = importlib.util.spec_from_file_location(
        "bench_for_test", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    got, source = bench.serving_set(3, path)
    assert source == path and _same(sts, got)
    with pytest.raises(SystemExit):
        bench.serving_set(4, path)


def test_size_lanes_keep_large_requests_off_the_small_lane_and_take_the_cheapest_first():
    """Three workers: two take small requests only, the third takes large ones first.  Every batch is
    ordered cheapest first (orbitals^3 x k-points), and every request completes."""
    sd = syn.default_shell_dict()
    norb = lambda st: sum(sum(2 * l + 1 for l in sd[int(z)]) for z in st["numbers"])
    taken, lock = [], threading.Lock()

    def fake_exec(structures, stream):
        w = server.workers.index(threading.current_thread())
        with lock:
            taken.append((w, [float(norb(st)) ** 3 * len(st["kpoints"]) for st in structures],
                          [norb(st) for st in structures]))
        time.sleep(0.005)
        return [{"eigenvalues": np.zeros(1), "band_gap_eV": 0.0} for _ in structures]

    rng = np.random.default_rng(5)
    sts = _structs(40, seed=5)
    for pos in (3, 11, 19, 30):                     # 40 atoms of Z = 21..30: 360 orbitals, above the 256 line
        st = syn.random_structure(rng, 40, zmax=30)
        st["numbers"] = 21 + (np.asarray(st["numbers"]) % 10)
        st["kpoints"] = np.zeros((2, 3))
        sts.insert(pos, st)
    server = SV.Server(FakeModel(), sd, device="cpu", mem_budget_bytes=1 << 40, n_workers=3, executor=fake_exec)
    assert server.small_workers == 2
    lat, wall, res = SV.poisson_stream(server, sts, rate=5000.0, seed=3)
    server.close()
    assert len(lat) == len(sts)
    assert sum(len(n) for _, _, n in taken) == len(sts)
    for w, cost, n in taken:
        if w < 2:
            assert max(n) <= 256
        assert cost == sorted(cost)
    assert any(max(n) > 256 for w, _, n in taken if w == 2)


def test_admission_counts_the_device_wide_scratch():
    """A request whose problems run on the device-wide eigensolver also holds that solver's scratch while in
    flight; below the threshold the estimate is H, S, eigenvalues and DOS alone."""
    import ctypes
    from slakonet_gb300 import _lib
    base = SV.request_bytes(1300, 5, 1000)
    assert SV.request_bytes(1300, 5, 1000, wide_threshold=2000) == base
    need = ctypes.c_int64(0)
    _lib.call("skn_eigh_wide_scratch_bytes", 5, 1300, ctypes.addressof(need))
    assert need.value > 0
    assert SV.request_bytes(1300, 5, 1000, wide_threshold=512) == base + need.value
