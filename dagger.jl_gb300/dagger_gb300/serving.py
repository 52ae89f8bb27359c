"""Continuous-batching solve server on one GPU.

Requests (an SPD matrix resident on the device, right-hand sides, a backward
error target) arrive over time.  The server

  * admits a request when a slot is free AND its device-memory footprint fits
    the HBM budget (free-HBM accounting: FP64 matrix 8n^2, packed FP32 factor
    ~2n^2, 16-bit panels, refinement vectors); otherwise it waits in the queue
    (first come, first served; a request larger than the whole budget is
    rejected);
  * runs admitted requests concurrently, each on its own CUDA stream and host
    worker, so their kernels overlap on the device; small systems (n <= 1024)
    that are waiting together are grouped into one persistent batched launch
    (dg_batched_potrs, FP32 factor + FP64 refinement);
  * keeps factors resident after a solve (LRU under the same budget), so a
    later request for the same matrix with new right-hand sides skips the
    factorization;
  * records arrival, start and completion times, reporting throughput and
    p50 / p99 latency (arrival -> solution on the device).

Each request's result is independent of what else is in flight: every
kernel a request uses reads only that request's data, in a fixed order, so a
request gives the same bits alone and in the mix (tests/test_gpu_serving.py).
"""
from __future__ import annotations

import math
import queue
import threading
import time
from dataclasses import dataclass, field

import torch

from .batched import PackedBatch, batched_solve_packed
from .darray import Blocks, DArray
from .mixed import MixedCholesky

SMALL_N = 1024


@dataclass
class Request:
    rid: int
    A: torch.Tensor | None          # n x n FP64 on the device (None when reusing a factor)
    B: torch.Tensor                 # n x r FP64 on the device
    matrix_id: int                  # factors are kept per matrix id
    precision: str = "bf16x3"
    tol: float = 1e-12
    arrival: float = 0.0
    start: float = 0.0
    done: float = 0.0
    X: torch.Tensor | None = None
    report: dict = field(default_factory=dict)
    error: str | None = None
    event: threading.Event = field(default_factory=threading.Event)

    @property
    def n(self):
        return int(self.B.shape[0])

    @property
    def nrhs(self):
        return int(self.B.shape[1]) if self.B.dim() == 2 else 1


def footprint_bytes(n, r, factored: bool) -> int:
    """Device bytes a request needs while it runs (factor included unless
    the factor is already resident)."""
    tiles = 8 * n * n
    factor = 0 if factored else (4 * (n * n // 2 + n * 1024) + 4 * n * 1024 + 8 * 1024 * 1024)
    vectors = 8 * n * r * 3 + 4 * n * r
    return tiles + factor + vectors


class Server:
    def __init__(self, budget_bytes: float = 150e9, slots: int = 8, nb: int = 512,
                 batch_small: bool = True, device=None):
        self.budget = int(budget_bytes)
        self.slots = slots
        self.nb = nb
        self.batch_small = batch_small
        self.device = torch.device(device or "cuda")
        self.q: "queue.Queue[Request | None]" = queue.Queue()
        self.lock = threading.Condition()
        self.in_use = 0
        self.active = 0
        self.resident: dict[int, tuple] = {}   # matrix_id -> (factor, DArray, bytes, last_used)
        self.pinned: dict[int, int] = {}       # matrix_id -> requests using its resident factor
        self.completed: list[Request] = []
        self.rejected: list[Request] = []
        self.t0 = time.perf_counter()
        self._stop = False
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(slots)]
        self.free_streams = list(range(slots))
        self.dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self.dispatcher.start()

    # -- client side ----------------------------------------------------------
    def now(self):
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        """Queues a request.  Its tensors may still be in flight on the
        submitting thread's current stream: the request's worker stream waits
        on an event recorded here before it reads them."""
        req.arrival = self.now()
        req._ready = torch.cuda.Event()
        req._ready.record(torch.cuda.current_stream(self.device))
        self.q.put(req)
        return req

    def close(self):
        self.q.put(None)
        self.dispatcher.join()
        with self.lock:
            while self.active:
                self.lock.wait()
        for f, _, _, _ in self.resident.values():
            f.close()
        self.resident.clear()

    # -- admission --------------------------------------------------------------
    def _resident_bytes(self):
        return sum(v[2] for v in self.resident.values())

    def _evict_for(self, need):
        """Drops least recently used resident factors that no running request
        uses until `need` more bytes fit the budget."""
        while self.in_use + self._resident_bytes() + need > self.budget:
            idle = [k for k in self.resident if not self.pinned.get(k)]
            if not idle:
                return
            victim = min(idle, key=lambda k: self.resident[k][3])
            f, _, _, _ = self.resident.pop(victim)
            f.close()

    def _admit(self, reqs):
        """Reserves memory and one stream slot for the group `reqs` (a single
        request, or small systems batched together); False if rejected."""
        with self.lock:
            need = 0
            for req in reqs:
                need += footprint_bytes(req.n, req.nrhs, req.matrix_id in self.resident)
            if need > self.budget:
                t = self.now()
                for req in reqs:
                    req.error = "larger than the HBM budget"
                    req.done = t
                    self.rejected.append(req)
                    req.event.set()
                return False
            while (self.active >= self.slots or
                   self.in_use + self._resident_bytes() + need > self.budget):
                self._evict_for(need)
                if (self.active < self.slots and
                        self.in_use + self._resident_bytes() + need <= self.budget):
                    break
                self.lock.wait()
            self.in_use += need
            self.active += 1
            lead = reqs[0]
            lead._need = need
            lead._stream = self.free_streams.pop()
            for req in reqs:
                if req.matrix_id in self.resident:
                    self.pinned[req.matrix_id] = self.pinned.get(req.matrix_id, 0) + 1
                    req._pinned = True
            return True

    def _release(self, req):
        with self.lock:
            self.in_use -= req._need
            self.active -= 1
            self.free_streams.append(req._stream)
            if getattr(req, "_pinned", False):
                self.pinned[req.matrix_id] -= 1
            self.lock.notify_all()

    # -- dispatch ---------------------------------------------------------------
    def _dispatch(self):
        pending = []
        closing = False
        while True:
            try:
                item = self.q.get(timeout=0.002 if pending else None)
                if item is None:
                    closing = True
                else:
                    pending.append(item)
                while True:   # drain everything that has arrived meanwhile
                    item = self.q.get_nowait()
                    if item is None:
                        closing = True
                    else:
                        pending.append(item)
            except queue.Empty:
                pass
            if pending:
                small = [r for r in pending if self.batch_small and r.n <= SMALL_N and
                         r.nrhs <= 8 and r.matrix_id not in self.resident and r.A is not None]
                large = [r for r in pending if r not in small]
                pending = []
                if small and self._admit(small):  # the group shares one slot
                    threading.Thread(target=self._run_batch, args=(small,), daemon=True).start()
                for req in large:
                    if self._admit([req]):
                        threading.Thread(target=self._run_one, args=(req,), daemon=True).start()
            if closing and not pending:
                return

    # -- workers ----------------------------------------------------------------
    def _run_one(self, req: Request):
        stream = self.streams[req._stream]
        try:
            req.start = self.now()
            stream.wait_event(req._ready)
            with torch.cuda.stream(stream):
                ent = self.resident.get(req.matrix_id)
                if ent is None:
                    DA = DArray.from_array(req.A, Blocks(self.nb, self.nb))
                    F = MixedCholesky(DA, req.precision, stream=stream)
                    fbytes = F.stats()["device_bytes"] + 8 * req.n * req.n
                else:
                    F, DA, fbytes, _ = ent
                X, rep = F.solve(req.B, tol=req.tol, stream=stream)
                stream.synchronize()
                req.X, req.report = X, rep
            with self.lock:
                self.resident[req.matrix_id] = (F, DA, fbytes, self.now())
        except Exception as e:  # reported per request, the server keeps going
            req.error = repr(e)
        finally:
            req.done = self.now()
            self._release(req)
            self.completed.append(req)
            req.event.set()

    def _run_batch(self, grp):
        lead = grp[0]
        stream = self.streams[lead._stream]
        try:
            t = self.now()
            for r in grp:
                r.start = t
                stream.wait_event(r._ready)
            with torch.cuda.stream(stream):
                P = PackedBatch([r.A for r in grp], [r.B.reshape(r.n, -1) for r in grp])
                rep = batched_solve_packed(P, "fp32_ir", tol=min(r.tol for r in grp),
                                           stream=stream)
                stream.synchronize()
            for i, r in enumerate(grp):
                r.X = P.solution(i).clone()
                r.report = {"batched": True, "group": len(grp),
                            "backward_error": rep["backward_error"][i],
                            "iterations": rep["iterations"][i], "info": rep["info"][i]}
                if rep["info"][i]:
                    r.error = f"not positive definite (info {rep['info'][i]})"
        except Exception as e:
            for r in grp:
                r.error = repr(e)
        finally:
            t = self.now()
            for r in grp:
                r.done = t
                self.completed.append(r)
                r.event.set()
            self._release(lead)


def latency_stats(reqs):
    lat = sorted((r.done - r.arrival) * 1e3 for r in reqs if r.error is None)
    if not lat:
        return {"p50_ms": None, "p99_ms": None, "count": 0}

    def pct(p):
        k = max(0, min(len(lat) - 1, int(math.ceil(p / 100.0 * len(lat))) - 1))
        return lat[k]
    return {"p50_ms": pct(50), "p99_ms": pct(99), "mean_ms": sum(lat) / len(lat),
            "count": len(lat)}


# ---------------------------------------------------------------------------
# synthetic request streams
# ---------------------------------------------------------------------------

class MatrixFactory:
    """Seeded SPD matrices A = Q diag(l) Q' (Q from the QR of a Gaussian, one
    per distinct order, computed in FP32 and cached; l log-spaced on
    [1, kappa]), built on the device and widened to FP64.  Matrices are
    cached by (n, kappa), so request streams drawn with the same seed at
    different arrival rates share their matrices."""

    def __init__(self, device, seed=0):
        self.device = torch.device(device)
        self.seed = seed
        self.q = {}
        self.mats = {}

    def Q(self, n):
        if n not in self.q:
            g = torch.Generator(device=self.device)
            g.manual_seed(self.seed * 100003 + n)
            G = torch.randn(n, n, generator=g, device=self.device, dtype=torch.float32)
            self.q[n] = torch.linalg.qr(G)[0]
        return self.q[n]

    def matrix(self, n, kappa):
        key = (n, kappa)
        if key in self.mats:
            return self.mats[key]
        Q = self.Q(n)
        lam = torch.logspace(0.0, math.log10(kappa), n, device=self.device, dtype=torch.float32)
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        A = ((Q * lam) @ Q.T).double()
        torch.backends.cuda.matmul.allow_tf32 = prev
        A = 0.5 * (A + A.T)
        self.mats[key] = A
        return A

    def drop_q(self):
        """Frees the cached orthogonal factors (the matrices stay)."""
        self.q.clear()


def make_workload(count, rate, seed=0, nlo=64, nhi=16384, klo=1e2, khi=1e6, rmax=64,
                  reuse=0.3, device="cuda", factory=None, round_to=64):
    """Poisson arrivals at `rate` per second: n log-uniform on [nlo, nhi]
    (rounded to a multiple of round_to), kappa log-uniform on [klo, khi],
    1..rmax right-hand sides, a fraction `reuse` of requests reusing an
    earlier matrix (a resident factor) with new right-hand sides.  The
    requests' contents depend on `seed` only and the arrival times on
    (seed, rate), so streams at different rates carry the same requests.
    Returns a list of (arrival offset in s, Request)."""
    import random
    rnd = random.Random(seed)
    arr = random.Random(f"arrivals:{seed}:{rate}")
    fac = factory or MatrixFactory(device, seed)
    t = 0.0
    out = []
    mats = []   # (matrix_id, A, kappa)
    for i in range(count):
        t += arr.expovariate(rate) if rate > 0 else 0.0
        if mats and rnd.random() < reuse:
            mid, A, kap = mats[rnd.randrange(len(mats))]
        else:
            n = math.exp(rnd.uniform(math.log(nlo), math.log(nhi)))
            n = max(round_to, int(round(n / round_to)) * round_to)
            kap = math.exp(rnd.uniform(math.log(klo), math.log(khi)))
            A = fac.matrix(n, kap)
            mid = len(mats)
            mats.append((mid, A, kap))
        n = A.shape[0]
        r = rnd.randint(1, rmax)
        g = torch.Generator(device=fac.device)
        g.manual_seed(seed * 7919 + i)
        B = torch.randn(n, r, generator=g, device=fac.device, dtype=torch.float64)
        prec = "bf16x3" if kap <= 1e6 else "fp32"
        out.append((t, Request(rid=i, A=A, B=B, matrix_id=mid, precision=prec)))
    return out


def run_workload(server, work, realtime=True):
    """Submits the requests at their arrival offsets and waits for all."""
    t0 = time.perf_counter()
    for t, req in work:
        if realtime:
            dt = t - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
        server.submit(req)
    for _, req in work:
        req.event.wait()
    return time.perf_counter() - t0
