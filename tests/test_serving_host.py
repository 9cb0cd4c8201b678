"""Host logic of the continuous-batching request loop, without a GPU:
admission against the HBM budget, slot limits, Poisson arrivals, latency
accounting, and a failing job not stopping the others (failure injected on
the host by the executor)."""
import threading
import time

import numpy as np

from pyloworder_gb300 import serving


def test_admission_respects_budget_and_slots():
    jobs = serving.make_mix(40, seed=3, m_range=(1000, 100000), n_range=(8, 64), rate=2000.0)
    active = {"n": 0, "max": 0}
    lock = threading.Lock()

    def executor(job, wid):
        with lock:
            active["n"] += 1
            active["max"] = max(active["max"], active["n"])
        time.sleep(0.001 + job.m * job.n * 1e-10)
        with lock:
            active["n"] -= 1
        return {"ok": job.jid}

    foot = lambda j: float(j.m * j.n * 4)  # noqa: E731
    budget = 3 * max(foot(j) for j in jobs)
    srv = serving.Server(hbm_budget_bytes=budget, slots=4, executor=executor, footprint=foot)
    done, summ = srv.run(jobs, realtime=True)
    assert summ["completed"] == 40 and summ["failed"] == 0
    assert active["max"] <= 4
    assert srv.peak_in_use <= budget
    assert all(j.done >= j.admitted >= j.arrival - 1e-6 for j in done)
    assert summ["p99_ms"] >= summ["p50_ms"] > 0
    assert {j.result["ok"] for j in done} == set(range(40))


def test_failed_and_oversized_jobs_do_not_stop_the_mix():
    jobs = serving.make_mix(12, seed=4, m_range=(1000, 5000), n_range=(8, 32))
    jobs.append(serving.Job(99, "POD", 10**9, 1000, seed=1))  # cannot fit

    def executor(job, wid):
        if job.jid == 5:
            raise RuntimeError("injected failure")
        return {"ok": True}

    srv = serving.Server(hbm_budget_bytes=1e9, slots=3, executor=executor,
                         footprint=lambda j: float(j.m * j.n * 4))
    done, summ = srv.run(jobs, realtime=False)
    by = {j.jid: j for j in done}
    assert by[5].error.startswith("RuntimeError")
    assert by[99].error == "exceeds the HBM budget"
    assert summ["completed"] == 11 and summ["failed"] == 1 and summ["rejected"] == 1


def test_mix_distribution():
    jobs = serving.make_mix(2000, seed=1, rate=100.0)
    m = np.array([j.m for j in jobs])
    n = np.array([j.n for j in jobs])
    assert m.min() >= 16384 and m.max() <= 4194304
    assert n.min() >= 32 and n.max() <= 1024
    kinds = {k: sum(j.kind == k for j in jobs) for k in ("POD", "DMD", "SPOD")}
    assert all(500 < v < 850 for v in kinds.values())
    gaps = np.diff([j.arrival for j in jobs])
    assert abs(gaps.mean() - 0.01) < 0.002  # Poisson at 100 jobs/s
