"""Continuous-batching request loop for POD / DMD / SPOD jobs on one GPU.

Jobs arrive over time (e.g. Poisson arrivals); each is a snapshot matrix of
its own size, generated on the device from its seed.  The server keeps up to
`slots` jobs in flight, one per CUDA stream, and admits the next arrived job
as soon as a slot is free AND its HBM footprint (input, workspace, outputs)
fits in the remaining budget; admitted jobs' kernels overlap on the device.
Latency = completion time - arrival time; the loop reports jobs/s and
p50 / p99 latency.  The work of each job is exactly the library call a user
makes (POD.run / DMD.run / SPOD.run on device tensors), so a job's result is
the same alone and in the mix.

There is no counterpart in pyLOM (it runs one analysis per MPI job).
"""
from __future__ import annotations

import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import DMD, POD, SPOD
from . import _lib as L
from . import datagen


@dataclass
class Job:
    jid: int
    kind: str      # "POD" | "DMD" | "SPOD"
    m: int
    n: int
    seed: int
    arrival: float = 0.0          # seconds after the start of the run
    admitted: float = math.nan
    done: float = math.nan
    result: dict = field(default_factory=dict)
    error: str = ""


def make_mix(njobs, seed=5, m_range=(16_384, 4_194_304), n_range=(32, 1024), rate=None,
             kinds=("POD", "DMD", "SPOD")):
    """Jobs with log-uniform m and n, uniform type and Poisson arrivals at
    `rate` jobs/s (all at t=0 when rate is None)."""
    rng = np.random.default_rng(seed)
    jobs = []
    t = 0.0
    for j in range(njobs):
        m = int(np.exp(rng.uniform(np.log(m_range[0]), np.log(m_range[1]))))
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        kind = kinds[int(rng.integers(len(kinds)))]
        if kind == "SPOD":
            n = max(n, 64)  # at least a few Welch blocks of nDFT >= 8
        if rate:
            t += rng.exponential(1.0 / rate)
        jobs.append(Job(j, kind, m, n, seed=10_000 + j, arrival=t))
    return jobs


def spod_nfft(n):
    """pyLOM's default block length 2^floor(log2(n/10)), clamped to >= 8."""
    return max(8, int(2 ** math.floor(math.log2(max(n / 10, 1)))))


def footprint_bytes(job, precision="mixed"):
    """HBM the job holds while in flight (input, mean-removed copy, outputs,
    workspace), from the library's own workspace queries."""
    lib = L.load()
    s = 4
    prec = L.PREC_MIXED if precision == "mixed" else L.PREC_FP64
    m, n = job.m, job.n
    base = 2 * s * m * n  # X and its mean-removed copy
    if job.kind == "POD":
        return base + s * m * n + lib.plom_tsqr_svd_workspace(L.F32, prec, m, n)
    if job.kind == "DMD":
        return base + 2 * s * m * n + lib.plom_tsqr_svd_workspace(L.F32, prec, m, n - 1)
    nfft = spod_nfft(n)
    nolap = nfft // 2
    nb = max(1, (n - nolap) // (nfft - nolap))
    nf = nfft // 2 + 1
    q = 2 * s * m * nb * nf
    return base + 2 * q + s * m * nb * nf + lib.plom_tsqr_svd_workspace(L.C64, prec, m, nb)


def generate(job):
    """The job's snapshot matrix on the current stream (FP32, POD-style field
    as config 1, per-job seed)."""
    nx, ny = datagen.grid_for_points(job.m)
    return datagen.pod_field_device(nx, ny, job.n, 10, seed=job.seed, noise=1e-4, amp_pow=None,
                                    dtype="float32", distinct=False, m=job.m, compute="float32")


def run_job(job, X, precision="mixed"):
    """Run one job on device data; returns a small summary on the host."""
    if job.kind == "POD":
        U, S, V = POD.run_device(X, X.shape[1], precision=precision)
        return {"S": S.double().cpu().numpy()}
    if job.kind == "DMD":
        r = min(10, job.n - 2)
        muR, muI, Phi, b = DMD.run_device(X, X.shape[1], r, precision=precision)
        return {"mu": (muR.double() + 1j * muI.double()).cpu().numpy(),
                "babs": b.abs().double().cpu().numpy()}
    t = np.arange(job.n, dtype=np.float64)
    nfft = spod_nfft(job.n)
    Lm, P, f = SPOD.run_device(X, X.shape[1], t, nDFT=nfft, precision=precision)
    return {"L0": Lm[:, 0].double().cpu().numpy(), "f": np.asarray(f)}


class Server:
    """Admission-controlled continuous batching over `slots` CUDA streams.

    `executor(job, stream_index)` runs one job and returns its result; the
    default generates the job's data and runs it on the worker's own CUDA
    stream.  `footprint(job)` gives the bytes a job holds while admitted.
    """

    def __init__(self, hbm_budget_bytes=150e9, slots=4, precision="mixed", executor=None,
                 footprint=None):
        self.budget = float(hbm_budget_bytes)
        self.slots = int(slots)
        self.precision = precision
        self.lock = threading.Condition()
        self.in_use = 0.0
        self.peak_in_use = 0.0
        self.free_slots = self.slots
        self.executor = executor
        self.footprint = footprint or (lambda j: footprint_bytes(j, self.precision))
        self._streams = {}
        # (job id, stream index, start event, end event) of every GPU job, recorded
        # on the job's stream: the device-side timeline of the mix (see timeline())
        self.events = []

    def _gpu_execute(self, job, wid):
        torch = L.torch()
        stream = self._streams.get(wid)
        if stream is None:
            stream = self._streams[wid] = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            X = generate(job)
            res = run_job(job, X, self.precision)
            del X
            ev1.record(stream)
        stream.synchronize()
        self.events.append((job.jid, wid, ev0, ev1))
        return res

    def timeline(self, ref):
        """[(job id, stream index, start ms, end ms)] of the GPU jobs, in ms
        after the CUDA event `ref` (recorded before the run), from the events
        each job recorded on its own stream."""
        return sorted((jid, wid, ref.elapsed_time(a), ref.elapsed_time(b))
                      for jid, wid, a, b in self.events)

    def _worker(self, wid, work_q, done_q, t0):
        execute = self.executor or self._gpu_execute
        while True:
            item = work_q.get()
            if item is None:
                return
            job, nbytes = item
            try:
                job.result = execute(job, wid)
            except Exception as e:  # a failing job reports its error; the others continue
                job.error = f"{type(e).__name__}: {e}"
            job.done = time.perf_counter() - t0
            with self.lock:
                self.in_use -= nbytes
                self.free_slots += 1
                self.lock.notify_all()
            done_q.put(job)

    def run(self, jobs, realtime=True):
        """Serve `jobs` (sorted by arrival).  Returns the finished jobs and a
        summary {jobs_per_s, p50_ms, p99_ms, ...}."""
        if self.executor is None:
            L.require_cuda()
            L.load()
        jobs = sorted(jobs, key=lambda j: j.arrival)
        sizes = [self.footprint(j) for j in jobs]
        work_q: queue.Queue = queue.Queue()
        done_q: queue.Queue = queue.Queue()
        t0 = time.perf_counter()
        workers = [threading.Thread(target=self._worker, args=(w, work_q, done_q, t0), daemon=True)
                   for w in range(self.slots)]
        for w in workers:
            w.start()
        rejected = []
        for job, nbytes in zip(jobs, sizes):
            if nbytes > self.budget:
                job.error = "exceeds the HBM budget"
                rejected.append(job)
                continue
            if realtime:
                wait = job.arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
            with self.lock:
                while self.free_slots == 0 or self.in_use + nbytes > self.budget:
                    self.lock.wait()
                self.free_slots -= 1
                self.in_use += nbytes
                self.peak_in_use = max(self.peak_in_use, self.in_use)
            if not realtime:
                job.arrival = time.perf_counter() - t0
            job.admitted = time.perf_counter() - t0
            work_q.put((job, nbytes))
        for _ in workers:
            work_q.put(None)
        for w in workers:
            w.join()
        if self.executor is None:
            L.torch().cuda.synchronize()
        finished = []
        while not done_q.empty():
            finished.append(done_q.get())
        wall = time.perf_counter() - t0
        ok = [j for j in finished if not j.error]
        lat = np.array([(j.done - j.arrival) * 1e3 for j in ok]) if ok else np.array([np.nan])
        summary = {"jobs": len(jobs), "completed": len(ok), "failed": len(finished) - len(ok),
                   "rejected": len(rejected), "wall_s": wall,
                   "jobs_per_s": len(ok) / wall if wall > 0 else float("nan"),
                   "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                   "slots": self.slots, "hbm_budget_gb": self.budget / 1e9,
                   "peak_admitted_gb": self.peak_in_use / 1e9, "precision": self.precision,
                   "errors": [(j.jid, j.kind, j.m, j.n, j.error) for j in finished if j.error][:8]}
        return finished + rejected, summary
