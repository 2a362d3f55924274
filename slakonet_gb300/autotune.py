"""Launch-shape autotuner for the batched eigensolver.

The library holds the eigensolver in three launch shapes (64, 128 and 256
threads per CTA, each with its own CTAs-per-SM, unroll and shared-memory
staging size; see ``build.EIG_SHAPES``).  ``autotune`` times every shape on
random Hermitian-definite problems at the upper edge of each problem-size
bucket and keeps the fastest; the result is cached as JSON per GPU and
library build.  ``Engine`` then runs each bucket's problems with its shape,
the groups on forked streams so they share the GPU.
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import json
import os
import statistics
import time
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr

SHAPES = ["", "_t32", "_t64", "_t256", "_blk"]  # export suffixes; "" is the 128-thread default, "_blk" the blocked one
BUCKETS = [16, 32, 64, 128, 256, 512, 1024, 2048]
# Untuned default: the blocked Cholesky and reduction above 128 orbitals, where it measured 18-20% faster
# on GB300 (n = 200-492); below, the unblocked kernel is faster (the panels are too short to pay).
BLOCKED_FROM_BUCKET = 256


class Tuning:
    def __init__(self, choice: Dict[int, str], timings: Optional[dict] = None):
        self.choice = {int(k): v for k, v in choice.items()}
        self.timings = timings or {}

    def shape_for(self, n: int) -> str:
        for u in BUCKETS:
            if n <= u:
                return self.choice.get(u, "")
        return ""

    def to_json(self) -> dict:
        return {"choice": {str(k): v for k, v in self.choice.items()}, "timings": self.timings}

    @classmethod
    def default(cls) -> "Tuning":
        """Untuned shapes: 128 threads up to 128 orbitals, the blocked shape from 256.  On the uneven batch
        this policy runs at 692-706 ms per eigensolve on GB300, run after run.  Policies that put the small
        problems on the 32- or 64-thread shapes are as fast at best but swing to 780-830 ms: their many
        small CTAs, launched beside the blocked shape on other streams, can take the SMs' slots first and
        delay the large problems, whose completion ends the step."""
        return cls({u: ("_blk" if u >= BLOCKED_FROM_BUCKET else "") for u in BUCKETS})


def _cache_key(device) -> str:
    props = torch.cuda.get_device_properties(device)
    lib = _lib.lib_path()
    h = hashlib.sha1(f"{props.name}|{props.multi_processor_count}|{os.path.getmtime(lib)}".encode()).hexdigest()[:16]
    return h


def default_cache_path() -> str:
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return os.environ.get("SKN_AUTOTUNE_CACHE", os.path.join(root, "_build", "autotune.json"))


def _problems(n: int, count: int, device, seed: int = 0):
    g = torch.Generator(device=device).manual_seed(seed)
    X = torch.randn(count, n, n, dtype=torch.complex128, device=device, generator=g)
    H = (X + X.mH) / 2
    Y = torch.randn(count, n, n, dtype=torch.complex128, device=device, generator=g) * 0.1
    S = torch.eye(n, dtype=torch.complex128, device=device) + Y @ Y.mH / n
    return H.transpose(1, 2).contiguous(), S.transpose(1, 2).contiguous()


def time_shape(suffix: str, n: int, count: int, device, reps: int = 2) -> float:
    H0, S0 = _problems(n, count, device)
    nv = torch.full((count,), n, dtype=torch.int32, device=device)
    off = torch.arange(count, dtype=torch.int64, device=device) * n * n
    eoff = torch.arange(count, dtype=torch.int64, device=device) * n
    order = torch.arange(count, dtype=torch.int32, device=device)
    eig = torch.empty(count * n, dtype=torch.float64, device=device)
    st = torch.empty(count, dtype=torch.int32, device=device)
    ctr = torch.zeros(2, dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    best = float("inf")
    for r in range(reps + 1):
        H = torch.view_as_real(H0.clone()).reshape(-1)
        S = torch.view_as_real(S0.clone()).reshape(-1)
        torch.cuda.synchronize(device)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        call("skn_eigh_gen_batched" + suffix, count, ptr(nv), ptr(off), ptr(eoff), ptr(order), ptr(H), ptr(S),
             ptr(eig), ptr(st), ptr(ctr), n, stream)
        b.record()
        torch.cuda.synchronize(device)
        if r:
            best = min(best, a.elapsed_time(b) * 1e-3)
    return best


def time_cluster(n: int, count: int, cluster: int, device, reps: int = 1) -> float:
    """Seconds for ``count`` random problems of n orbitals on the cluster eigensolver
    (``cluster`` CTAs per problem); cluster 0 times the one-CTA-per-problem kernel."""
    H0, S0 = _problems(n, count, device)
    nv = torch.full((count,), n, dtype=torch.int32, device=device)
    off = torch.arange(count, dtype=torch.int64, device=device) * n * n
    eoff = torch.arange(count, dtype=torch.int64, device=device) * n
    order = torch.arange(count, dtype=torch.int32, device=device)
    eig = torch.empty(count * n, dtype=torch.float64, device=device)
    st = torch.empty(count, dtype=torch.int32, device=device)
    ctr = torch.zeros(2, dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    scratch, need = None, ctypes.c_int64(0)
    if cluster:
        call("skn_eigh_large_scratch_bytes", count, n, cluster, ctypes.addressof(need))
        scratch = torch.empty(max(need.value // 8, 1), dtype=torch.float64, device=device)
    best = float("inf")
    for _ in range(reps):
        H = torch.view_as_real(H0.clone()).reshape(-1)
        S = torch.view_as_real(S0.clone()).reshape(-1)
        torch.cuda.synchronize(device)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        if cluster:
            call("skn_eigh_gen_large", count, ptr(nv), ptr(off), ptr(eoff), ptr(order), ptr(H), ptr(S), ptr(eig),
                 ptr(st), ptr(ctr), ptr(scratch), need.value, n, cluster, stream)
        else:
            call("skn_eigh_gen_batched", count, ptr(nv), ptr(off), ptr(eoff), ptr(order), ptr(H), ptr(S), ptr(eig),
                 ptr(st), ptr(ctr), n, stream)
        b.record()
        torch.cuda.synchronize(device)
        best = min(best, a.elapsed_time(b) * 1e-3)
    if int((st != 0).sum()):
        raise _lib.SknError("random test problems failed to solve")
    return best


def buckets_up_to(max_n: int) -> List[int]:
    """The buckets a batch whose largest problem has ``max_n`` orbitals uses."""
    out = [u for u in BUCKETS if u < max_n]
    nxt = [u for u in BUCKETS if u >= max_n]
    return out + nxt[:1]


def autotune(device="cuda", cache: Optional[str] = None, budget_s: float = 0.04, use_cache: bool = True,
             buckets: Optional[List[int]] = None) -> Tuning:
    """Fastest shape per bucket (cached per GPU and library build); buckets not tuned keep the default."""
    device = torch.device(device)
    _lib.load()
    cache = cache or default_cache_path()
    key = _cache_key(device)
    if use_cache and os.path.exists(cache):
        try:
            data = _read_cache(cache)
            want = set(buckets or BUCKETS)
            if key in data and want <= {int(k) for k in data[key]["choice"]}:
                return Tuning(data[key]["choice"], data[key].get("timings"))
        except (OSError, ValueError, KeyError):
            pass
    choice, timings = {}, {}
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    for u in (buckets or BUCKETS):
        flops = 32.0 / 3.0 * u ** 3
        # about budget_s of work at the FP64 rate, at least one problem per SM
        count = int(min(20000, max(sms, budget_s * 0.8e12 / flops)))
        reps = 2 if u <= 512 else 1
        t = {sfx: time_shape(sfx, u, count, device, reps) for sfx in SHAPES}
        choice[u] = min(t, key=t.get)
        timings[str(u)] = {(sfx or "_t128"): round(v * 1e3, 3) for sfx, v in t.items()}
    tun = Tuning(choice, timings)
    try:
        tun = _merge_into_cache(cache, key, tun)
    except (OSError, ValueError, KeyError):
        pass
    return tun


def _read_cache(path: str) -> dict:
    with open(path) as f:
        return json.load(f)


def _merge_into_cache(path: str, key: str, tun: Tuning) -> Tuning:
    """Merge ``tun`` with the buckets tuned earlier under ``key`` and write the cache through a
    temporary file, so a reader never sees a partly written file.  Returns the merged tuning."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    data = _read_cache(path) if os.path.exists(path) else {}
    if key in data:
        merged = {int(k): v for k, v in data[key]["choice"].items()}
        merged.update(tun.choice)
        mt = dict(data[key].get("timings", {}))
        mt.update(tun.timings)
        tun = Tuning(merged, mt)
    data[key] = tun.to_json()
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1)
    os.replace(tmp, path)
    return tun


def candidate_policies(tuning: Optional[Tuning] = None) -> List[Tuning]:
    """Whole-batch candidates: the untuned default (128 threads below 256 orbitals, blocked from 256) and
    the blocked shape from 128.  Policies with the 32- or 64-thread shapes for the small buckets, or the
    per-bucket winners of ``autotune`` (``tuning``, timed one shape at a time), are not offered: beside the
    blocked launch on other streams their many small CTAs make the step swing between 690 and 830 ms.
    ``tuning`` is accepted for its per-bucket timings only."""
    del tuning
    return [Tuning.default(), Tuning({u: ("_blk" if u >= 128 else "") for u in BUCKETS})]


def tune_batch(engine, db, candidates: Optional[List[Tuning]] = None, reps: int = 3) -> Tuning:
    """Time the eigensolve of the batch itself under each candidate policy; return the one with the
    smallest median over ``reps`` trials (the groups of a policy run concurrently on several streams, and
    some policies vary from run to run with the order in which their CTAs reach the SMs).

    H(k) and S(k) are built once and cloned per trial (the eigensolver works in place)."""
    candidates = candidates or candidate_policies()
    dev = engine.device
    base = engine.execute(db, keep_hs=True, hs_only=True)
    plan = db.plan
    n_prob = len(plan.prob_n)
    eig = torch.empty(max(plan.eig_total, 1), dtype=torch.float64, device=dev)
    st = torch.empty(max(n_prob, 1), dtype=torch.int32, device=dev)
    ctr = torch.zeros(2, dtype=torch.int32, device=dev)
    saved = engine.tuning
    best, best_t = None, float("inf")
    timings = []
    try:
        for cand in candidates:
            engine.tuning = cand
            trials = []
            for _ in range(reps):
                H = base.H.clone()
                S = base.S.clone()
                torch.cuda.synchronize(dev)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                engine._eig_values(db, H, S, eig, st, ctr, torch.cuda.current_stream(dev).cuda_stream)
                b.record()
                torch.cuda.synchronize(dev)
                trials.append(a.elapsed_time(b) * 1e-3)
            tbest = statistics.median(trials)
            timings.append(round(tbest * 1e3, 2))
            if tbest < best_t:
                best, best_t = cand, tbest
    finally:
        engine.tuning = saved
    best.timings = dict(best.timings)
    best.timings["batch_trials_ms"] = timings
    return best


def main(argv=None):
    ap = argparse.ArgumentParser(description="Time the eigensolver kernels on random Hermitian-definite problems.")
    ap.add_argument("--n", type=int, nargs="+", default=[1024], help="orbitals per problem")
    ap.add_argument("--count", type=int, default=1, help="problems per launch")
    ap.add_argument("--clusters", type=int, nargs="+", default=[16],
                    help="CTAs per problem on the cluster eigensolver; 0 = one-CTA-per-problem kernel")
    ap.add_argument("--reps", type=int, default=1)
    args = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    _lib.load()
    out = {}
    for n in args.n:
        for c in args.clusters:
            out[f"n{n}_c{c}"] = round(time_cluster(n, args.count, c, dev, args.reps), 6)
    print(json.dumps({"count": args.count, "seconds": out}))


if __name__ == "__main__":
    main()
