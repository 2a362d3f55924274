"""Continuous-batching server for the properties path.

Requests (one periodic structure each) arrive at any time.  A request is
admitted when its device-memory estimate fits the budget left by requests
already admitted; admitted requests wait in a queue.  Each worker thread owns
a CUDA stream: it takes requests that are admitted and not yet started
(up to ``max_batch_problems`` (structure, k) problems), plans them as one
batch, runs the whole path on its stream, copies the results to the host and
releases their memory.  With two or more workers, a batch formed from
requests that arrived while another batch was on the GPU runs concurrently
with it, so arrivals never wait for a whole batch to drain.

Latency under load comes from small requests waiting behind large ones: a
batch ends only when its largest eigensolve ends.  So requests are sorted
into two lanes by orbital count (``large_orbitals``).  ``small_workers`` of
the workers take small requests only; the others take large requests first
and small ones when no large one waits.  Within a lane a worker takes the
cheapest requests first (n^3 x k-points), and problems above
``wide_threshold`` orbitals run on the device-wide eigensolver (every SM on
one structure's k-points), which shortens the longest eigensolve of a batch.

The reference serves one structure per call (slakonet/optim.py:949-1075 via
predict_slakonet.py); there is no queue, batch or stream there.
"""
from __future__ import annotations

import concurrent.futures as cf
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np
import torch

from . import engine as E
from .model import MultiElementSkfParameterOptimizer, properties_dict

MAX_N = E.LARGE_MAX_N   # cluster eigensolver bound (csrc/eigh_cluster.cu)


def request_bytes(n_orb: int, nk: int, dos_points: int, wide_threshold: Optional[int] = None) -> int:
    """Device bytes one request holds while in flight (H, S, eigenvalues, DOS, slack for bonds), plus the
    device-wide eigensolver's scratch when its problems are above ``wide_threshold`` orbitals (panels,
    partial sums and the tensor-core update's integer slices: about 5.5 KB per orbital and k-point)."""
    nb = int(2 * 16 * n_orb * n_orb * nk + 8 * n_orb * nk + 8 * dos_points + (8 << 20))
    if wide_threshold is not None and wide_threshold < n_orb <= MAX_N and nk > 0:
        import ctypes
        from . import _lib
        need = ctypes.c_int64(0)
        _lib.call("skn_eigh_wide_scratch_bytes", nk, n_orb, ctypes.addressof(need))
        nb += int(need.value)
    return nb


@dataclass
class Request:
    rid: int
    structure: dict
    n_orb: int
    nk: int
    nbytes: int
    t_submit: float
    future: cf.Future = field(default_factory=cf.Future)
    t_start: float = 0.0
    t_done: float = 0.0


class Admission:
    """Memory-budget admission (host-side, thread-safe)."""

    def __init__(self, budget_bytes: int):
        self.budget = int(budget_bytes)
        self.used = 0
        self.lock = threading.Lock()

    def try_admit(self, nbytes: int) -> bool:
        with self.lock:
            if self.used + nbytes <= self.budget or self.used == 0:
                self.used += nbytes
                return True
            return False

    def release(self, nbytes: int):
        with self.lock:
            self.used -= nbytes


class Server:
    """Continuous-batching front end of ``MultiElementSkfParameterOptimizer``."""

    def __init__(self, model: MultiElementSkfParameterOptimizer, shell_dict: Dict[int, List[int]], device="cuda",
                 species: Optional[Sequence[int]] = None, mem_budget_bytes: Optional[int] = None,
                 n_workers: int = 2, max_batch_problems: int = 8192, dos_range=(-20.0, 10.0),
                 dos_points: int = 1000, dos_sigma: float = 0.1, dos_window: float = 9.0,
                 executor: Optional[Callable] = None, large_orbitals: Optional[int] = 256,
                 small_workers: Optional[int] = None, large_threshold: Optional[int] = 512,
                 wide_threshold: Optional[int] = 512):
        self.model = model
        self.sd = shell_dict
        self.device = torch.device(device)
        self.dos = dict(dos_range=dos_range, dos_points=dos_points, dos_sigma=dos_sigma, dos_window=dos_window)
        self.max_batch_problems = max_batch_problems
        # size lanes: requests above large_orbitals are "large"; the first small_workers workers take
        # small requests only (None: all but one worker when there are at least two; no lanes when
        # large_orbitals is None)
        self.large_orbitals = large_orbitals
        if large_orbitals is None:
            small_workers = 0
        elif small_workers is None:
            small_workers = n_workers - 1 if n_workers >= 2 else 0
        self.small_workers = max(0, min(int(small_workers), n_workers - 1))
        self.large_threshold = large_threshold
        self.wide_threshold = wide_threshold
        if mem_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            mem_budget_bytes = int(0.6 * free)
        self.adm = Admission(mem_budget_bytes)
        self.tables = model.table_set(shell_dict, self.device, species) if executor is None else None
        if self.tables is not None:
            torch.cuda.synchronize(self.device)   # tables are read by every worker stream
        self.executor = executor or self._execute
        self.pending: "queue.Queue[Request]" = queue.Queue()     # submitted, not admitted
        self.ready: List[Request] = []                            # admitted, not started
        self.cv = threading.Condition()
        self.stop = False
        self.closing = False
        self.rid = 0
        self.workers = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(n_workers)]
        self.admitter = threading.Thread(target=self._admit_loop, daemon=True)
        self.batches = 0
        self.rejected = 0
        for w in self.workers:
            w.start()
        self.admitter.start()

    # ------------------------------------------------------------ clients
    def submit(self, structure: dict) -> cf.Future:
        zs = np.asarray(structure["numbers"]).reshape(-1)
        missing = sorted({int(z) for z in zs} - set(int(z) for z in self.sd))
        n_orb = sum(sum(2 * l + 1 for l in self.sd[int(z)]) for z in zs) if not missing else 0
        nk = len(structure["kpoints"])
        with self.cv:
            self.rid += 1
            req = Request(self.rid, structure, n_orb, nk,
                          request_bytes(n_orb, nk, self.dos["dos_points"], self.wide_threshold), time.perf_counter())
        err = None
        if missing:
            err = ValueError(f"no shells for element Z={missing[0]}")
        elif n_orb > MAX_N:
            err = ValueError(f"{n_orb} orbitals exceed the eigensolver's {MAX_N}")
        else:
            try:   # a malformed structure is refused alone instead of failing the batch it would join
                E.check_structure(structure)
            except ValueError as e:
                err = e
        with self.cv:
            if err is None and self.closing:
                err = RuntimeError("the server is closed")
            if err is None:
                self.pending.put(req)      # under the lock, so close() cannot slip in between
                return req.future
            self.rejected += 1
        req.future.set_exception(err)
        return req.future

    def close(self):
        """Refuse new requests, finish every request already submitted, then stop the threads."""
        with self.cv:
            if self.closing:
                return
            self.closing = True
        self.pending.put(None)             # the admitter admits everything queued before this, then exits
        self.admitter.join()
        with self.cv:
            self.stop = True               # workers exit once the ready list is empty
            self.cv.notify_all()
        for w in self.workers:
            w.join()

    # ------------------------------------------------------------ internals
    def _admit_loop(self):
        waiting: Optional[Request] = None
        while True:
            if waiting is None:
                waiting = self.pending.get()
                if waiting is None:
                    return
            if self.adm.try_admit(waiting.nbytes):
                with self.cv:
                    self.ready.append(waiting)
                    self.cv.notify()
                waiting = None
            else:
                time.sleep(0.0005)
                with self.cv:
                    if self.stop:
                        return

    def is_large(self, r: Request) -> bool:
        return self.large_orbitals is not None and r.n_orb > self.large_orbitals

    def _take_batch(self, worker: int = -1) -> List[Request]:
        """The requests of a worker's next batch: its lane's ready requests, cheapest first (n^3 x nk),
        up to max_batch_problems problems.  A small-lane worker takes small requests only; any other
        worker takes large requests when one waits, else small ones."""
        small_only = 0 <= worker < self.small_workers
        with self.cv:
            while True:
                if small_only:
                    cand = [r for r in self.ready if not self.is_large(r)]
                else:
                    cand = [r for r in self.ready if self.is_large(r)] or list(self.ready)
                if cand or self.stop:
                    break
                self.cv.wait(0.05)
            if not cand:
                return []
            cand.sort(key=lambda r: (float(r.n_orb) ** 3 * r.nk, r.rid))
            batch, probs = [], 0
            for r in cand:
                if batch and probs + r.nk > self.max_batch_problems:
                    break
                probs += r.nk
                batch.append(r)
            taken = {id(r) for r in batch}
            self.ready = [r for r in self.ready if id(r) not in taken]
            return batch

    def _execute(self, structures, stream):
        with torch.cuda.stream(stream):
            eng = E.Engine(self.tables, stream=stream, large_threshold=self.large_threshold,
                           wide_threshold=self.wide_threshold)
            plan = E.plan_batch(structures, self.tables)
            db = E.DeviceBatch(plan, self.device)
            res = eng.execute(db, **self.dos)
            eng.check_tables()
            out = []
            eig = res.eig.to("cpu", non_blocking=False)
            dos = res.dos.to("cpu")
            stats = res.stats.to("cpu")
            mu = res.mu.to("cpu")
            status = res.eig_status.to("cpu")
            for s in range(plan.n_struct):
                o, nk, nb = int(plan.eig_off_struct[s]), int(plan.nk[s]), int(plan.nb[s])
                ok = status[plan.prob_struct == s]
                out.append({"eigenvalues": eig[o:o + nk * nb].view(nk, nb), "dos": dos[s], "stats": stats[s],
                            "fermi_energy_Ha": float(mu[s]), "band_gap_eV": float(stats[s, E.STAT["gap_ev"]]),
                            "eig_status_ok": bool((ok == 0).all())})
            return out

    def _worker(self, idx: int):
        stream = torch.cuda.Stream(self.device) if self.executor == self._execute else None
        while True:
            batch = self._take_batch(idx)
            if not batch:
                with self.cv:
                    if self.stop and not self.ready:
                        return
                    if self.stop and idx < self.small_workers:
                        return           # what is left is large: a worker of the other lane takes it
                continue
            # claim each future: one a client cancelled while it waited is dropped here (its memory
            # released), and none can be cancelled once its batch runs
            live = []
            for r in batch:
                if r.future.set_running_or_notify_cancel():
                    live.append(r)
                else:
                    self.adm.release(r.nbytes)
            batch = live
            if not batch:
                continue
            t0 = time.perf_counter()
            for r in batch:
                r.t_start = t0
            try:
                outs = self.executor([r.structure for r in batch], stream)
                err = None
            except Exception as e:   # surfaced on every request of the batch
                outs, err = None, e
            t1 = time.perf_counter()
            with self.cv:
                self.batches += 1
            for i, r in enumerate(batch):
                r.t_done = t1
                self.adm.release(r.nbytes)
                if err is not None:
                    r.future.set_exception(err)
                else:
                    res = outs[i]
                    res["latency_s"] = t1 - r.t_submit
                    r.future.set_result(res)


def poisson_stream(server: Server, structures: Sequence[dict], rate: float, seed: int = 0):
    """Submit ``structures`` with exponential inter-arrival times (mean 1/rate); wait for all.

    Returns (latencies_s [array], wall_s, results)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(structures))
    t0 = time.perf_counter()
    due = t0
    futs = []
    for st, gsec in zip(structures, gaps):
        due += gsec
        now = time.perf_counter()
        if due > now:
            time.sleep(due - now)
        futs.append(server.submit(st))
    results = []
    for f in futs:
        try:
            results.append(f.result())
        except Exception as e:   # rejected requests
            results.append({"error": str(e)})
    wall = time.perf_counter() - t0
    lat = np.array([r["latency_s"] for r in results if "latency_s" in r])
    return lat, wall, results
