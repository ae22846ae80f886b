"""Job server scheduling logic on the CPU, with a stand-in backend that only counts steps.

Checks what continuous batching promises independently of the GPU: every job runs exactly
its own number of steps (finished jobs leave a batch while the rest runs on), jobs are never
admitted before they arrive, the device memory budget, the batch-slot limit and the
systems-per-batch limit hold at every moment, batches never mix plugin kinds, and a job that
can never fit is rejected instead of blocking the queue.
"""
import threading
import time

import numpy as np
import pytest

from lpmd2_gb300 import inputs as I
from lpmd2_gb300.serve import JobResult, Server, footprint, summarize


class CountingBackend:
    def __init__(self, step_seconds=2e-6):
        self.step_seconds = step_seconds
        self.lock = threading.Lock()
        self.open_batches = 0
        self.max_open = 0
        self.kinds_per_batch = []
        self.sizes = []
        self.live_bytes = 0
        self.peak_bytes = 0

    def list_radius(self, kind):
        return 8.8 if kind == "lj" else 7.7

    def open(self, kind, systems):
        h = dict(kind=kind, n=len(systems), done=[0] * len(systems), active=[True] * len(systems),
                 bytes=footprint(systems, self.list_radius(kind)), systems=systems)
        with self.lock:
            self.open_batches += 1
            self.max_open = max(self.max_open, self.open_batches)
            self.kinds_per_batch.append({s["kind"] for s in systems})
            self.sizes.append(len(systems))
            self.live_bytes += h["bytes"]
            self.peak_bytes = max(self.peak_bytes, self.live_bytes)
        return h

    def device_bytes(self, h):
        return h["bytes"]

    def advance(self, h, n):
        assert n > 0
        for k in range(h["n"]):
            if h["active"][k]:
                h["done"][k] += n
        time.sleep(n * self.step_seconds)

    def read(self, h, k):
        return np.zeros((1, 3)), np.zeros((1, 3)), {"steps_done": h["done"][k]}

    def retire(self, h, k):
        assert h["active"][k]
        h["active"][k] = False

    def close(self, h):
        with self.lock:
            self.open_batches -= 1
            self.live_bytes -= h["bytes"]


def fake_system(job):
    n = 4 * job["k"] ** 3
    a = 5.72 if job["kind"] == "lj" else 3.61
    return dict(kind=job["kind"], natoms=n, L=np.full(3, job["k"] * a))


def small_jobs(n, rate, seed=5):
    jobs = I.job_stream(n, rate, seed=seed, nmin=500, nmax=20000, smin=100, smax=2000)
    return jobs


def check_results(jobs, results, backend, server):
    assert [r.id for r in results] == [j["id"] for j in jobs]
    for j, r in zip(jobs, results):
        assert isinstance(r, JobResult)
        if r.error:
            continue
        assert r.thermo["steps_done"] == j["steps"]
        assert r.admitted >= j["arrival"] - 1e-9
        assert r.finished >= r.admitted
    assert server.peak_used <= server.budget
    assert backend.peak_bytes <= server.budget
    assert backend.max_open <= server.max_batches
    assert max(backend.sizes) <= server.max_systems
    assert all(len(k) == 1 for k in backend.kinds_per_batch)
    assert backend.open_batches == 0 and abs(server.used) < 1e-6


@pytest.mark.parametrize("rate", [50.0, 500.0])
def test_all_jobs_run_their_own_steps(rate):
    jobs = small_jobs(40, rate)
    be = CountingBackend()
    srv = Server(be, budget_bytes=150e9, max_batches=4, max_systems=8, chunk_steps=700)
    t0 = time.monotonic()
    res = srv.serve(jobs, fake_system)
    s = summarize(res, time.monotonic() - t0)
    check_results(jobs, res, be, srv)
    assert s["completed"] == 40 and s["rejected"] == 0
    assert s["p99_latency_s"] >= s["p50_latency_s"] > 0


def test_tight_budget_serialises_but_completes():
    jobs = small_jobs(24, 1000.0, seed=7)
    sizes = [footprint([fake_system(j)], 8.8) for j in jobs]
    budget = 1.5 * max(sizes)  # about one big job at a time
    be = CountingBackend()
    srv = Server(be, budget_bytes=budget, max_batches=8, max_systems=64)
    res = srv.serve(jobs, fake_system)
    check_results(jobs, res, be, srv)
    assert all(r.error is None for r in res)
    assert srv.batches_started > 1


def test_job_larger_than_budget_is_rejected():
    jobs = small_jobs(10, 200.0, seed=9)
    sizes = [footprint([fake_system(j)], 8.8) for j in jobs]
    big = int(np.argmax(sizes))
    budget = (sorted(sizes)[-1] + sorted(sizes)[-2]) / 2  # only the largest cannot fit
    be = CountingBackend()
    srv = Server(be, budget_bytes=budget, max_batches=2, max_systems=4)
    res = srv.serve(jobs, fake_system)
    check_results(jobs, res, be, srv)
    assert res[big].error is not None
    assert all(r.error is None for k, r in enumerate(res) if k != big)


def test_size_classes_never_share_a_batch():
    jobs = small_jobs(30, 1000.0, seed=11)
    be = CountingBackend()
    srv = Server(be, budget_bytes=150e9, max_batches=8, max_systems=64, small_atoms=5000)
    res = srv.serve(jobs, fake_system)
    check_results(jobs, res, be, srv)
    by_batch = {}
    for r in res:
        by_batch.setdefault(r.batch, set()).add((r.kind, r.natoms < 5000))
    assert all(len(v) == 1 for v in by_batch.values())


def test_backend_failure_surfaces():
    class Failing(CountingBackend):
        def advance(self, h, n):
            raise RuntimeError("device error")

    jobs = small_jobs(4, 100.0)
    srv = Server(Failing(), budget_bytes=150e9, max_batches=2)
    with pytest.raises(RuntimeError, match="device error"):
        srv.serve(jobs, fake_system)
    assert srv.used == pytest.approx(0.0)


def test_lanes_follow_the_live_atoms():
    from lpmd2_gb300.serve import lanes_for

    assert [lanes_for(n) for n in (500, 999, 1_000, 9_999, 10_000, 59_999, 60_000, 3_000_000)] == \
        [16, 16, 4, 4, 2, 2, 1, 1]


def test_work_order_admits_shortest_first_within_the_atom_limit():
    """order="work" with max_batch_atoms: every batch holds at most the limit (or one larger
    job alone), all jobs still run their own steps, and a backlog is admitted shortest first:
    the job with the least atoms x steps goes into the first batch, and the first batch's jobs
    are shorter on average than the last batch's."""
    jobs = [dict(j, arrival=0.0) for j in small_jobs(40, 50.0)]  # one backlog at t = 0
    be = CountingBackend()
    srv = Server(be, budget_bytes=150e9, max_batches=1, max_systems=64, order="work", max_batch_atoms=40000)
    results = srv.serve(jobs, fake_system)
    check_results(jobs, results, be, srv)
    work = {}
    atoms = {}
    for j, r in zip(jobs, results):
        work.setdefault(r.batch, []).append(4 * j["k"] ** 3 * j["steps"])
        atoms.setdefault(r.batch, []).append(4 * j["k"] ** 3)
    for b in atoms:
        assert sum(atoms[b]) <= 40000 or len(atoms[b]) == 1
    order = sorted(work)  # batch ids are given in admission order
    assert len(order) > 2
    least = min(4 * j["k"] ** 3 * j["steps"] for j in jobs)
    assert least in work[order[0]]
    assert np.mean(work[order[0]]) < np.mean(work[order[-1]])


def test_unknown_admission_order_is_rejected():
    with pytest.raises(ValueError, match="admission order"):
        Server(CountingBackend(), order="random")
