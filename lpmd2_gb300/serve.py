"""Job server: MD jobs that arrive over time, run as continuously formed batches on one GPU.

Each job is one independent system (an LPMD run: atoms, plugins, a number of steps).  The
scheduler admits waiting jobs whenever a batch slot and device memory are free: it packs the
waiting jobs of one kind (same plugins) into a new gbmd batch, which runs on its own CUDA
stream and host thread beside the batches already on the GPU, so work of jobs that arrived
at different times overlaps on the device.  Inside a batch every advance runs to the next job
completion (or a chunk bound); a finished job is read back and deactivated
(gbmd_batch_set_active), and the rest of the batch runs on without it.  When every job of a
batch is done the batch is destroyed and its memory returns to the budget.

Admission is against a byte budget: a batch is admitted on an estimate of its footprint
(`footprint`), and once created its actual device bytes replace the estimate in the ledger.
A job whose own footprint exceeds the whole budget is rejected.

The backend is duck-typed (``GbmdBackend`` below drives libgbmd); tests drive the same
scheduler with a CPU stand-in.
"""
from __future__ import annotations

import dataclasses
import math
import threading
import time
from typing import Callable

import numpy as np

# Device bytes per atom that do not depend on the list: FP64 state, double-buffered
# positions and gather copies, permutation scratch, cell arrays and per-atom bookkeeping.
BASE_BYTES_PER_ATOM = 640
LIST_BYTES_PER_ENTRY = 4


@dataclasses.dataclass
class JobResult:
    id: int
    kind: str
    natoms: int
    steps: int
    arrival: float
    admitted: float = math.nan
    finished: float = math.nan
    batch: int = -1
    pos: np.ndarray | None = None
    vel: np.ndarray | None = None
    thermo: dict | None = None
    error: str | None = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def list_capacity(natoms: int, L, rl: float) -> int:
    """Per-atom list capacity the engine allocates for one system (its sizing rule)."""
    vol = float(L[0]) * float(L[1]) * float(L[2])
    expect = 4.18879 * rl ** 3 * natoms / vol
    return (int(math.ceil(expect * 1.35)) + 32 + 7) & ~7


def footprint(systems: list[dict], rl: float) -> int:
    """Estimated device bytes of one batch holding `systems` (list capacity is batch-wide)."""
    n = sum(int(s["natoms"]) for s in systems)
    cap = max(list_capacity(int(s["natoms"]), s["L"], rl) for s in systems)
    return int(n * (BASE_BYTES_PER_ATOM + LIST_BYTES_PER_ENTRY * cap))


class Server:
    def __init__(self, backend, budget_bytes: float = 150e9, max_batches: int = 4, max_systems: int = 512,
                 chunk_steps: int = 5000, window_s: float = 0.2, fill_atoms: int = 2_000_000,
                 small_atoms: int = 0, order: str = "arrival", max_batch_atoms: int = 0,
                 clock: Callable[[], float] = time.monotonic):
        """window_s / fill_atoms: a batch is formed once its oldest waiting job has waited
        window_s, or once fill_atoms atoms of its class are waiting (enough to fill the GPU),
        so that jobs arriving close together share a batch instead of each taking a slot.

        order: the order in which the waiting jobs of the chosen class go into a new batch:
        "arrival", "work" (least atoms x steps first) or "steps" (fewest steps first, so that a
        batch's jobs end close together).  max_batch_atoms: atoms one batch
        takes at most (0: no limit; a single larger job still gets a batch of its own).  A batch
        holds its slot until its longest job is done, so with "work" and a limit, batches of
        short jobs turn their slots over quickly and a backlog is served shortest first.

        small_atoms: jobs below this size form their own batches (0: off, the default).  A
        batch steps in lockstep, so a small job with many steps sharing a batch with large
        systems advances at their step time.  Measured on GB300 with the default stream, the
        split did not pay: each extra class takes a batch slot, and a small batch's kernels
        still wait for SM slots behind the large batches' running blocks."""
        self.backend = backend
        self.small_atoms = int(small_atoms)
        if order not in ("arrival", "work", "steps"):
            raise ValueError(f"unknown admission order {order!r}")
        self.order = order
        self.max_batch_atoms = int(max_batch_atoms)
        self.window_s = float(window_s)
        self.fill_atoms = int(fill_atoms)
        self.budget = float(budget_bytes)
        self.max_batches = int(max_batches)
        self.max_systems = int(max_systems)
        self.chunk_steps = int(chunk_steps)
        self.clock = clock
        self.used = 0.0
        self.peak_used = 0.0
        self.batches_started = 0
        self._cv = threading.Condition()
        self._running: dict[int, threading.Thread] = {}
        self._errors: list[BaseException] = []

    # ------------------------------------------------------------------ scheduler
    def serve(self, jobs: list[dict], materialize: Callable[[dict], dict]) -> list[JobResult]:
        """Runs `jobs` (dicts with id, kind, steps, arrival in seconds from the start) to
        completion; `materialize(job)` gives its system (pos, vel, mass, Z, L, natoms).

        The systems are the requests' payloads, which clients bring with them: they are made
        before the clock starts, and a job enters the queue at its arrival time."""
        systems = {j["id"]: materialize(j) for j in jobs}
        t0 = self.clock()
        now = lambda: self.clock() - t0  # noqa: E731
        future = sorted(jobs, key=lambda j: (j["arrival"], j["id"]))
        waiting: list[tuple[dict, dict]] = []
        results: dict[int, JobResult] = {}
        with self._cv:
            while True:
                t = now()
                while future and future[0]["arrival"] <= t:
                    job = future.pop(0)
                    system = systems[job["id"]]
                    res = JobResult(job["id"], job["kind"], int(system["natoms"]), int(job["steps"]),
                                    job["arrival"])
                    results[job["id"]] = res
                    if footprint([system], self.backend.list_radius(job["kind"])) > self.budget:
                        res.error = "job footprint exceeds the whole device memory budget"
                        res.admitted = res.finished = t
                        continue
                    waiting.append((job, system))
                if self._errors:
                    # stop admitting; surface the failure once every running batch has ended
                    if not self._running:
                        raise self._errors[0]
                else:
                    self._admit(waiting, results, now)
                    if not future and not waiting and not self._running:
                        break
                timeout = 0.05
                if future:
                    timeout = min(timeout, future[0]["arrival"] - now())
                if waiting:
                    timeout = min(timeout, min(j["arrival"] for j, _ in waiting) + self.window_s - now())
                self._cv.wait(max(0.0, timeout))
        if self._errors:
            raise self._errors[0]
        return [results[j["id"]] for j in jobs]

    def _admit(self, waiting, results, now):
        while waiting and len(self._running) < self.max_batches:
            # the kind whose oldest job is ready: waited out the window, or enough atoms queued
            cls = None
            for c in dict.fromkeys(self._class(j, s) for j, s in waiting):
                ofc = [(j, s) for j, s in waiting if self._class(j, s) == c]
                oldest = min(j["arrival"] for j, _ in ofc)
                if now() - oldest >= self.window_s or sum(int(s["natoms"]) for _, s in ofc) >= self.fill_atoms:
                    cls = c
                    break
            if cls is None:
                return
            kind = cls[0]
            rl = self.backend.list_radius(kind)
            picked: list[tuple[dict, dict]] = []
            candidates = [(j, s) for j, s in waiting if self._class(j, s) == cls]
            if self.order == "work":
                candidates.sort(key=lambda js: (int(js[1]["natoms"]) * int(js[0]["steps"]), js[0]["arrival"]))
            elif self.order == "steps":
                candidates.sort(key=lambda js: (int(js[0]["steps"]), int(js[1]["natoms"]), js[0]["arrival"]))
            atoms = 0
            for job, system in candidates:
                if len(picked) >= self.max_systems:
                    break
                n = int(system["natoms"])
                if self.max_batch_atoms and picked and atoms + n > self.max_batch_atoms:
                    continue
                trial = [s for _, s in picked] + [system]
                if self.used + footprint(trial, rl) <= self.budget:
                    picked.append((job, system))
                    atoms += n
            if not picked:
                return  # the oldest kind does not fit yet: wait for memory
            for p in picked:
                waiting.remove(p)
            est = footprint([s for _, s in picked], rl)
            self.used += est
            self.peak_used = max(self.peak_used, self.used)
            bid = self.batches_started
            self.batches_started += 1
            t = now()
            for job, _ in picked:
                results[job["id"]].admitted = t
                results[job["id"]].batch = bid
            th = threading.Thread(target=self._run_batch, args=(bid, kind, picked, est, results, now), daemon=True)
            self._running[bid] = th
            th.start()

    def _class(self, job, system) -> tuple[str, bool]:
        """Batching class: plugin kind and whether the system is small."""
        return job["kind"], int(system["natoms"]) < self.small_atoms

    # ------------------------------------------------------------------ one batch
    def _run_batch(self, bid, kind, picked, est, results, now):
        held = est
        handle = None
        try:
            handle = self.backend.open(kind, [s for _, s in picked])
            real = self.backend.device_bytes(handle)
            with self._cv:
                self.used += real - held
                held = real
                self.peak_used = max(self.peak_used, self.used)
            remaining = [int(job["steps"]) for job, _ in picked]
            active = set(range(len(picked)))
            while active:
                n = min(min(remaining[k] for k in active), self.chunk_steps)
                self.backend.advance(handle, n)
                for k in active:
                    remaining[k] -= n
                for k in sorted(k for k in active if remaining[k] == 0):
                    pos, vel, thermo = self.backend.read(handle, k)
                    r = results[picked[k][0]["id"]]
                    r.pos, r.vel, r.thermo = pos, vel, thermo
                    r.finished = now()
                    active.discard(k)
                    if active:
                        self.backend.retire(handle, k)
        except BaseException as e:  # surfaced by serve()
            with self._cv:
                self._errors.append(e)
        finally:
            if handle is not None:
                try:
                    self.backend.close(handle)
                except BaseException as e:
                    with self._cv:
                        self._errors.append(e)
            with self._cv:
                self.used -= held
                self._running.pop(bid, None)
                self._cv.notify_all()


def partition(costs, world: int) -> list[list[int]]:
    """Indices of independent work items (systems or jobs) split over `world` GPUs by
    estimated cost (atoms x steps): longest first onto the least loaded rank.  Deterministic,
    so every rank computes the same split without an exchange."""
    loads = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-float(costs[k]), k)):
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(p) for p in parts]


def summarize(results: list[JobResult], wall_s: float) -> dict:
    ok = [r for r in results if r.error is None]
    lat = np.array([r.latency for r in ok]) if ok else np.array([math.nan])
    work = sum(r.natoms * r.steps for r in ok)
    return {"jobs": len(results), "completed": len(ok), "rejected": len(results) - len(ok),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "atom_steps": int(work), "wall_s": wall_s, "atom_steps_per_s": work / wall_s if wall_s > 0 else math.nan}


# ---------------------------------------------------------------------- libgbmd backend
def lanes_for(live_atoms: int) -> int:
    """Lanes per atom of the LJ force pass for a batch with this many live atoms: below about
    60k atoms one lane per atom leaves the GPU partly idle.  Thresholds from GB300 timings of
    single LJ liquids at rc 2.5 sigma (ms/step with 1/2/4/8/16 lanes: 864 atoms 0.046/0.040/
    0.036/0.035/0.034; 4,000: 0.051/0.043/0.040/0.039/0.043; 16,384: 0.047/0.039/0.041/0.047/
    0.062; 55,296: 0.055/0.055/0.065/0.089/0.141; 256,000: 0.140/0.163/0.203/0.319/0.566).
    Forces are the same for every choice, so changing it never changes a job's trajectory."""
    if live_atoms < 1_000:
        return 16
    if live_atoms < 10_000:
        return 4
    if live_atoms < 60_000:
        return 2
    return 1


class GbmdBackend:
    """Runs batches through libgbmd (mixed precision, Verlet lists, 10-step graph blocks)."""

    def __init__(self, device: int = 0, precision: str = "mixed", graph_block: int = 10, lj_skin_sigma: float = 0.3,
                 sc_skin: float = 0.5, small_atoms: int = 100_000):
        from . import gbmd
        from . import inputs as I

        self.gbmd, self.I = gbmd, I
        self.device = device
        self.precision = precision
        self.graph_block = graph_block
        self.small_atoms = small_atoms
        sigma = I.LJ_AR["sigma"]
        self.lj = dict(rc=2.5 * sigma, skin=lj_skin_sigma * sigma,
                       dt=0.005 * I.lj_reduced_units(sigma, I.LJ_AR["epsilon"], I.LJ_AR["mass"])["tau_fs"])
        self.sc = dict(rc=2.0 * I.SC_CU["a"], skin=sc_skin, dt=2.0)

    def list_radius(self, kind: str) -> float:
        p = self.lj if kind == "lj" else self.sc
        return p["rc"] + p["skin"]

    def plugins(self, kind: str):
        g, I = self.gbmd, self.I
        if kind == "lj":
            p = self.lj
            pot = g.Plugin("lennardjones", f"sigma {I.LJ_AR['sigma']} epsilon {I.LJ_AR['epsilon']} cutoff {p['rc']!r}")
        else:
            p = self.sc
            c = I.SC_CU
            pot = g.Plugin("suttonchen", f"e {c['e']} a {c['a']} n {c['n']} m {c['m']} c {c['c']} cutoff {p['rc']!r}")
        cm = g.Plugin("verletlist", f"cutoff {p['rc']!r} skin {p['skin']!r} maxneighbors 512")
        return cm, pot, g.Plugin("velocityverlet", f"dt {p['dt']!r}")

    def open(self, kind: str, systems: list[dict]):
        b = self.gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems], device=self.device)
        for k, s in enumerate(systems):
            b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        cm, pot, integ = self.plugins(kind)
        b.set_cell_manager(cm)
        b.add_potential(pot)
        b.set_integrator(integ)
        b.set_precision(self.precision)
        b.set_option("graph_block", self.graph_block)
        b.live = [int(s["natoms"]) for s in systems]
        b.high = False
        b.kind = kind
        b.lanes = 1
        self._prioritise(b)
        b.update_forces()
        return b

    def _prioritise(self, b):
        """Small batches run at the highest stream priority: their short kernels then take SM
        slots ahead of pending blocks of a large batch's kernels, instead of queueing behind
        them for every dependent launch of a step."""
        if not b.high and sum(b.live) <= self.small_atoms:
            b.set_option("stream_priority", 1)
            b.high = True
        lanes = lanes_for(sum(b.live)) if b.kind == "lj" and self.precision == "mixed" else 1
        if lanes != b.lanes:
            b.set_option("lanes_per_atom", lanes)
            b.lanes = lanes

    def device_bytes(self, b) -> int:
        return int(b.stats()["device_bytes"])

    def advance(self, b, n: int):
        b.do_steps(n)

    def read(self, b, k: int):
        pos, vel, _ = b.atoms(k)
        return pos, vel, b.thermo(k)

    def retire(self, b, k: int):
        b.set_active(k, False)
        b.live[k] = 0
        self._prioritise(b)

    def close(self, b):
        b.close()
