"""Benchmark of the MD timestep on GB300: atom-steps/s of the mixed-precision Verlet-list step
against the plain FP64 GPU path, for the single large Lennard-Jones liquid (FCC 40^3 = 256,000
atoms at rho* = 0.8442, melted at T* = 1.5, cutoff 2.5 sigma, Verlet skin 0.3 sigma rebuilt on
max displacement > skin/2, dt* = 0.005).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbmd|reference]

Prints one JSON line.  One process per GPU (torchrun for N > 1): every rank advances its own
replica of the system (the single-system path has no exchange step: "replicas only"); the
timed region is bracketed by a barrier and device synchronisation, and the slowest rank's
time is used.  --impl reference times the reference algorithm on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SIGMA, EPS, MASS = 3.405, 0.0103, 39.948
RHO_STAR, T_STAR = 0.8442, 1.5
GRAPH_BLOCK = 10
# Bytes one mixed LJ step moves per atom: the Verlet-list entries it reads (about 88 x 4 B at
# rc + skin = 2.8 sigma), the FP32 gather copy (16 B read, 16 B written), positions (24 B read,
# 24 B written), velocities and accelerations (48 B read, 48 B written), the FP64 gather copy
# (32 B written), mass/forcefactor/flags (17 B) and the displacement reference (16 B): ~590 B,
# 151 MB at 256,000 atoms, larger than GB300's 129 MB L2.
WORKING_SET_NOTE = ("not flushed: inputs larger than L2 -- a step streams ~590 B per atom (Verlet list ~350 B, "
                    "FP64 state and gather copies), 151 MB at 256,000 atoms, against the 129 MB L2; value and "
                    "e2e are timed alike")


def workload(ncell: int = 40, seed: int = 2):
    from lpmd2_gb300 import inputs as I

    a = (4.0 / RHO_STAR) ** (1.0 / 3.0) * SIGMA
    pos, L = I.fcc_fast(ncell, ncell, ncell, a)
    pos = I.jitter(pos, 0.05 * SIGMA, seed=seed)
    m = np.full(len(pos), MASS)
    T = T_STAR * EPS / I.KBOLTZMANN
    vel = I.maxwell_boltzmann(m, T, seed=seed)
    tau = I.lj_reduced_units(SIGMA, EPS, MASS)["tau_fs"]
    return dict(pos=pos, L=L, vel=vel, mass=m, T=T, dt=0.005 * tau, rc=2.5 * SIGMA, skin=0.3 * SIGMA,
                natoms=len(pos), ncell=ncell)


def make_sim(w, precision: str, device: int = 0):
    from lpmd2_gb300 import gbmd

    sim = gbmd.Simulation(w["natoms"], w["L"], device=device)
    sim.set_atoms(w["pos"], w["vel"], Z=18, mass=w["mass"])
    sim.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {w['rc']!r} skin {w['skin']!r} maxneighbors 256"))
    sim.add_potential(gbmd.Plugin("lennardjones", f"sigma {SIGMA} epsilon {EPS} cutoff {w['rc']!r}"))
    sim.set_integrator(gbmd.Plugin("velocityverlet", f"dt {w['dt']!r}"))
    sim.set_precision(precision)
    sim.set_option("graph_block", GRAPH_BLOCK)
    return sim


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v: float) -> float:
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_model() -> str:
    """The host CPU's name (lscpu, else /proc/cpuinfo; Arm parts by their part number)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        info = Path("/proc/cpuinfo").read_text()
        for line in info.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
        parts = {"0xd4f": "Neoverse-V2", "0xd40": "Neoverse-V1", "0xd0c": "Neoverse-N1"}
        for line in info.splitlines():
            if line.startswith("CPU part"):
                return parts.get(line.split(":", 1)[1].strip(), "Arm part " + line.split(":", 1)[1].strip())
    except OSError:
        pass
    return platform.machine()


def cpu_sample(seconds_target: float = 15.0, procs: int | None = None) -> dict:
    """Times the reference CPU algorithm (oracle/_ref where built, else the C restatement) on
    a bounded sample: a 4,000-atom cut of the same liquid (FCC 10^3 at rho* 0.8442, T* 1.5,
    same cutoff), linkedcell + velocityverlet, one replica per host core."""
    import multiprocessing as mp

    ncores = procs or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(ncores) as pool:
        res = pool.map(_cpu_worker, [seconds_target] * ncores)
    steps = sum(r[0] for r in res)
    atoms = res[0][1]
    wall = max(r[2] for r in res)
    kind = res[0][3]
    # (i) one process on one core, next to (ii) one replica per core above
    with ctx.Pool(1) as pool:
        one = pool.map(_cpu_worker, [seconds_target / 2])[0]
    return {"value": steps * atoms / wall, "unit": "atom-steps/s", "cores": ncores, "kind": kind,
            "single_core_value": one[0] * one[1] / one[2], "cpu_model": cpu_model(),
            "sample": f"{ncores} replicas x {steps // ncores} steps of a {atoms}-atom cut of the liquid "
                      f"(FCC 10^3, linkedcell nx 4, velocityverlet, 2 force evaluations per step as the "
                      f"reference does), {wall:.1f} s; single_core_value: one process on one core"}


def _cpu_worker(budget: float):
    sys.path.insert(0, str(ROOT))
    import oracle
    from lpmd2_gb300 import inputs as I

    w = workload(ncell=10)
    n = w["natoms"]
    rc = w["rc"]
    cm_args = f"cutoff {rc!r} nx 4 ny 4 nz 4"
    pots = [("lennardjones", f"sigma {SIGMA} epsilon {EPS} cutoff {rc!r}", -1, -1)]
    if oracle.reference_available():
        kind = "reference"
        run = lambda k: oracle.run_reference(w["pos"], w["L"], "Ar", w["vel"], "linkedcell", cm_args, pots, w["dt"], k)
    else:
        kind = "port"
        run = lambda k: oracle.run_port(w["pos"], w["L"], np.full(n, 18), w["mass"], w["vel"], "linkedcell",
                                        cm_args, pots, w["dt"], k)
    t0 = time.perf_counter()
    run(1)
    t1 = time.perf_counter()
    run(3)
    t3 = time.perf_counter()
    per_step = max((t3 - t1) - (t1 - t0), 0.5 * (t1 - t0)) / 2.0  # without the set-up cost
    k = max(2, int(budget / max(per_step, 1e-4)))
    t0 = time.perf_counter()
    run(k)
    dt = time.perf_counter() - t0
    return (k, n, dt, kind)


def run_reference_arm(args):
    rank, world, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    w = workload()
    t0 = time.perf_counter()
    cb = cpu_sample(seconds_target=float(os.environ.get("GBMD_CPU_SECONDS", "12")))
    out = {
        "metric": "atom-steps/s", "value": cb["value"], "unit": "atom-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * w["natoms"] / cb["value"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": "lj_liquid_fcc40_256k", "natoms": w["natoms"], "precision": "fp64",
                   "sampled_as": cb["sample"]},
        "cpu_baseline": {"value": cb["value"], "unit": cb["unit"], "cores": cb["cores"], "kind": cb["kind"],
                         "sample": cb["sample"], "single_core_value": cb["single_core_value"],
                         "cpu_model": cb["cpu_model"]},
        "e2e": {"value": cb["value"], "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gbmd", choices=["gbmd", "reference"])
    ap.add_argument("--melt", type=int, default=2000,
                    help="untimed FP64 steps that melt the lattice into the common start (--profile: mixed steps)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--profile", action="store_true",
                    help="short direct-launch run of the workload for ncu (no timing, no JSON)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"], help="with --profile")
    ap.add_argument("--workload", default="lj", choices=["lj", "eam", "ensemble", "ensemble-small"],
                    help="with --profile: the LJ liquid, the Sutton-Chen copper, the 512-system ensemble, or 512 "
                         "systems of 256 atoms (FCC 4^3, the ensemble's smallest size)")
    ap.add_argument("--drift-steps", type=int, default=10000, help="NVE steps of the drift comparison")
    ap.add_argument("--batch-steps", type=int, default=100, help="timed steps of the batched ensemble (0: skip)")
    ap.add_argument("--eam-steps", type=int, default=100, help="timed steps of the Sutton-Chen Cu system (0: skip)")
    ap.add_argument("--eam-drift-steps", type=int, default=5000,
                    help="NVE steps of the Sutton-Chen drift comparison, both paths (0: skip)")
    ap.add_argument("--serve-jobs", type=int, default=200, help="jobs of the served stream (0: skip)")
    ap.add_argument("--budget-burst", type=int, default=80,
                    help="2,048,000-atom jobs of the burst that presses the 150 GB budget (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=100.0, help="Poisson arrival rate, jobs/s")
    ap.add_argument("--serve-sweep", default="10,100,500",
                    help="arrival rates (jobs/s) of the latency sweep, comma-separated ('' to skip; one GPU only)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.profile:
        run_profile(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local, dist = dist_setup(args.gpus)
    import torch

    from lpmd2_gb300 import gbmd

    torch.cuda.set_device(local)
    w = workload()
    N = w["natoms"]
    # the common start of every measurement: the jittered lattice melted by the plain FP64 path
    w_melt = w
    if args.melt:
        melt = make_sim(w, "fp64", device=local)
        melt.update_forces()
        melt.do_steps(args.melt)
        p_melt, v_melt, _ = melt.atoms()
        melt.close()
        w_melt = dict(w, pos=p_melt, vel=v_melt)
    sim = make_sim(w_melt, "mixed", device=local)
    sim.update_forces()
    # at least one whole graph block: the CUDA graph of a block is captured at its first use,
    # which must not fall inside the timed region
    sim.do_steps(max(args.warmup, GRAPH_BLOCK))
    sim.synchronize()

    def timed_steps(s, k):
        """k steps in ONE call (the library launches its 10-step graphs back to back), CUDA
        events on the simulation's stream around it.  No L2 flush: a step streams more than the
        129 MB L2 holds (WORKING_SET_NOTE), the same treatment as the end-to-end run."""
        st = torch.cuda.ExternalStream(s.stream, device=local)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s.do_steps(k)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1)

    def busy(s, seconds):
        """Untimed steps of the same work for about `seconds` (nvidia-smi samples every 200 ms, a
        20-step timed region lasts a few ms: the samples around it describe its clocks)."""
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            s.do_steps(GRAPH_BLOCK * 10)
            s.synchronize()

    with ClockSampler(local) as clk:
        busy(sim, 0.7)
        stats0 = sim.stats()
        barrier(dist)
        torch.cuda.synchronize()
        ms = timed_steps(sim, args.steps)
        torch.cuda.synchronize()
        barrier(dist)
        stats1 = sim.stats()
        busy(sim, 0.4)
    ms = allmax(dist, ms)
    value = N * args.steps * world / (ms * 1e-3)

    # plain FP64 GPU path on the same (melted) state
    sim64 = make_sim(w_melt, "fp64", device=local)
    sim64.update_forces()
    k64 = max(GRAPH_BLOCK, (args.steps // 5) // GRAPH_BLOCK * GRAPH_BLOCK)
    sim64.do_steps(GRAPH_BLOCK)
    ms64 = timed_steps(sim64, k64)
    value64 = N * k64 / (ms64 * 1e-3)

    # error of the mixed forces against FP64 at identical positions
    simm = make_sim(w_melt, "mixed", device=local)
    simm.update_forces()
    sim64b = make_sim(w_melt, "fp64", device=local)
    sim64b.update_forces()
    am = simm.atoms()[2]
    a64 = sim64b.atoms()[2]
    frel = float(np.sqrt(np.sum((am - a64) ** 2) / np.sum(a64 ** 2)))
    e_m, e_64 = simm.thermo()["potential_energy"], sim64b.thermo()["potential_energy"]
    w_m, w_64 = simm.thermo()["virial"], sim64b.thermo()["virial"]
    del simm, sim64b

    # kernel timing pass (direct launches, events around the force kernel on its stream)
    kt = kernel_times(w_melt, local)

    # end to end through the public API with pinned host buffers: upload the state, run a
    # 100-step chunk, read back the per-step thermo and the final state
    e2e = end_to_end(w_melt, local)

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_kind = "measured" if "hbm_gbs" in peaks else "fallback"
    # the fused force kernel moves the step's whole compulsory state once: read x, v, a
    # (72 B), write a, v, x (72 B), plus the force read of x counted by the 168 B/atom-step
    # convention (x is read once here)
    force_bytes_per_atom = 168.0
    achieved = force_bytes_per_atom * N / (kt["force_ms"] * 1e-3) / 1e9 if kt["force_ms"] else None
    traffic = profiled_traffic("k_force32_lj_liquid_256k.md")
    step_bytes_per_atom = 168.0
    step_achieved = step_bytes_per_atom * N * args.steps / (ms * 1e-3) / 1e9

    drift_cmp = measure_drift(w_melt, local, args.drift_steps) if args.drift_steps > 0 else None
    eam = eam_metal(local, args.eam_steps, args.eam_drift_steps) if args.eam_steps > 0 else None
    batched = batched_ensemble(local, args.batch_steps, rank=rank, world=world, dist=dist) if args.batch_steps > 0 else None
    served = served_stream(local, args.serve_jobs, args.serve_rate, rank, world, dist) if args.serve_jobs > 0 else None
    sweep = []
    sc_rate = sc_batched_rate(local) if args.serve_jobs > 0 and world == 1 else None
    burst = budget_burst(local, args.budget_burst) if args.budget_burst > 0 and world == 1 else None
    if args.serve_jobs > 0 and args.serve_sweep.strip() and world == 1:
        for rate in (float(x) for x in args.serve_sweep.split(",")):
            r = served if rate == args.serve_rate else served_stream(local, args.serve_jobs, rate, rank, world, dist)
            sweep.append({"rate_jobs_per_s": rate, "p50_latency_s": r["p50_latency_s"],
                          "p99_latency_s": r["p99_latency_s"], "atom_steps_per_s": r["atom_steps_per_s"],
                          "wall_s": r["wall_s"], "completed": r["completed"]})

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        cpu = cpu_sample(seconds_target=float(os.environ.get("GBMD_CPU_SECONDS", "12")))
    launches = stats1["kernel_launches"] - stats0["kernel_launches"]
    out = {
        "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64 (f64 integrate)",
        "data": "synthetic",
        "config": {"workload": "lj_liquid_fcc40_256k", "natoms": N, "rho_star": RHO_STAR, "T_star": T_STAR,
                   "cutoff_sigma": 2.5, "skin_sigma": 0.3, "dt_fs": w["dt"], "precision": "mixed",
                   "graph_block": GRAPH_BLOCK, "melt_steps": args.melt, "melt_precision": "fp64", "seed": 2,
                   "rng": "SplitMix64 (lpmd2_gb300/inputs.py)",
                   "l2": WORKING_SET_NOTE,
                   "warmup_note": "at least one 10-step graph block untimed (the graph is captured there), "
                                  "and about 1 s of untimed steps of the same work around the timed region "
                                  "while nvidia-smi samples the clocks",
                   "parallelism": f"replicas x{world}"},
        "ns_per_day": value / N / world * w["dt"] * 86400 * 1e-6,
        "gpu_launches": launches,
        "list_rebuilds_timed": stats1["list_rebuilds"] - stats0["list_rebuilds"],
        # details first; the driver keeps the end of the line, where the summary and the
        # contract's objects sit
        "batched": batched,
        "served": served,
        "served_sweep": sweep or None,
        "served_budget_burst": burst,
        "sc_batched": sc_rate,
        "eam": eam,
        "drift": drift_cmp,
        "kernel_ms": kt,
        "step_roofline": {"achieved": step_achieved, "peak": peak, "unit": "GB/s", "frac": step_achieved / peak,
                          "bytes_per_atom_step": step_bytes_per_atom},
        "flop_roofline": flop_roofline(value / world, RHO_STAR, clk.summary()),
        "fp64_value": value64 * world, "fp64_ms_per_step": ms64 / k64,
        "force_rms_rel_err_vs_fp64": frel, "epot_rel_err_vs_fp64": abs(e_m - e_64) / abs(e_64),
        "virial_rel_err_vs_fp64": abs(w_m - w_64) / abs(w_64),
        "speedup_vs_fp64": value / (value64 * world),
        "summary": summarize_line(value, value64 * world, e2e, frel, abs(e_m - e_64) / abs(e_64),
                                  abs(w_m - w_64) / abs(w_64), drift_cmp, eam, batched, served, sc_rate, burst),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "traffic": traffic,
                     "traffic_source": "not measured in this run: dram__bytes_read.sum + dram__bytes_write.sum "
                                       "of one ncu capture, read from profiles/k_force32_lj_liquid_256k.md; the "
                                       "Verlet list dominates it",
                     "kernel": "k_force32<pair> (fused LJ force + velocity kick + drift)",
                     "bytes_per_atom": force_bytes_per_atom, "launch_ms": kt["force_ms"],
                     "peak_source": peak_kind},
        "e2e": e2e,
        "clocks": clk.summary(),
    }
    if cpu:
        out["cpu_baseline"] = cpu
    print(json.dumps(out))


def summarize_line(value, value64, e2e, frel, erel, wrel, drift, eam, batched, served, sc_rate=None,
                   burst=None) -> dict:
    """The benchmark's headline figures in one short object: the mixed/FP64 ratio with its
    errors for each workload, NVE drift, and the served stream's latency against the batched
    engine's throughput."""
    r = lambda x, d=4: None if x is None else float(f"{x:.{d}g}")  # noqa: E731
    out = {"lj_mixed_over_fp64": r(value / value64), "lj_e2e_atom_steps_per_s": r(e2e["value"]),
           "lj_errors_vs_fp64": {"force_rms": r(frel, 3), "epot": r(erel, 3), "virial": r(wrel, 3)}}
    if drift:
        out["lj_drift_ev_per_atom_per_ns"] = {"mixed": r(drift["mixed_ev_per_atom_per_ns"], 3),
                                             "fp64": r(drift["fp64_ev_per_atom_per_ns"], 3), "ns": r(drift["ns"], 3)}
    if eam:
        out["eam_mixed_over_fp64"] = r(eam["speedup_vs_fp64"])
        out["eam_atom_steps_per_s"] = r(eam["value"])
        for key, tag in (("errors_20_fp64_steps", "eam_errors_20_steps"), ("errors_after_timed_run", "eam_errors_bench_state")):
            e = eam[key]
            out[tag] = {"force_rms": r(e["force_rms_rel_err_vs_fp64"], 3), "epot": r(e["epot_rel_err_vs_fp64"], 3),
                        "virial_pressure": r(e["virial_pressure_rel_err_vs_fp64"], 3)}
        if eam.get("drift"):
            d = eam["drift"]
            out["eam_drift_ev_per_atom_per_ns"] = {"mixed": r(d["mixed_ev_per_atom_per_ns"], 3),
                                                  "fp64": r(d["fp64_ev_per_atom_per_ns"], 3), "ns": r(d["ns"], 3)}
    if batched:
        out["ensemble_mixed_over_fp64"] = r(batched["speedup_vs_fp64"])
        out["ensemble_atom_steps_per_s"] = r(batched["value"])
    if served:
        out["served"] = {"p50_s": r(served["p50_latency_s"], 3), "p99_s": r(served["p99_latency_s"], 3),
                         "atom_steps_per_s": r(served["atom_steps_per_s"]), "jobs": served["completed"]}
        if batched and sc_rate:
            # the batched engine's rate for the same work: LJ at the ensemble's rate, copper at the
            # copper batch's, weighted by the stream's atom-steps of each kind
            wk = served["atom_steps_by_kind"]
            ideal = (wk["lj"] + wk["sc"]) / (wk["lj"] / batched["value"] + wk["sc"] / sc_rate["value"])
            out["served"]["batched_rate_same_mix"] = r(ideal)
            out["served"]["fraction_of_batched_same_mix"] = r(served["atom_steps_per_s"] / ideal, 3)
    if burst:
        out["budget_burst"] = {"peak_gb": r(burst["peak_budget_used_bytes"] / 1e9, 4), "jobs": burst["completed"],
                               "batches": burst["batches"]}
    return out


def run_profile(args):
    """The workload with direct launches only (graph_mode 0), for ncu: melt, warm up, then
    --steps steps.  Every kernel of a step is a separate launch on the simulation's stream.
    --workload eam profiles the Sutton-Chen copper system instead of the LJ liquid."""
    if args.workload in ("ensemble", "ensemble-small"):
        from lpmd2_gb300 import inputs as I

        if args.workload == "ensemble":
            systems = I.lj_ensemble(512, seed=4)
        else:
            systems = [I.lj_system(4, 0.70 + 0.25 * (q % 7) / 6, 0.7 + 1.3 * (q % 5) / 4, seed=900 + q)
                       for q in range(512)]
        b = make_batch(systems, args.precision, 0, {"skin_sigma": 0.3, "cell_scale": 1, "lanes_per_atom": 1})
        b.set_option("graph_mode", 0)
        b.update_forces()
        b.do_steps(args.melt + args.warmup)
        b.do_steps(args.steps)
        b.synchronize()
        print(json.dumps({"profile": True, "workload": args.workload, "systems": len(systems),
                          "natoms": sum(q["natoms"] for q in systems), "steps": args.steps, **b.stats()}))
        return
    if args.workload == "eam":
        sim, natoms = make_eam_sim(args.precision)
        sim.set_option("graph_mode", 0)
        sim.update_forces()
        sim.do_steps(args.melt + args.warmup)
        sim.do_steps(args.steps)
        sim.synchronize()
        print(json.dumps({"profile": True, "workload": "eam", "natoms": natoms, "steps": args.steps, **sim.stats()}))
        return
    w = workload()
    sim = make_sim(w, args.precision)
    sim.set_option("graph_mode", 0)
    sim.update_forces()
    sim.do_steps(args.melt + args.warmup)
    sim.do_steps(args.steps)
    sim.synchronize()
    print(json.dumps({"profile": True, "natoms": w["natoms"], "steps": args.steps, **sim.stats()}))


def kernel_times(w, device: int) -> dict:
    """Average device time per launch of each kernel class, from CUDA events the library
    records on its own stream around every launch (direct-launch mode)."""
    sim = make_sim(w, "mixed", device=device)
    sim.set_option("graph_mode", 0)
    sim.set_option("time_kernels", 1)
    sim.update_forces()
    sim.do_steps(50)
    st = sim.kernel_times()
    return st


def end_to_end(w, device: int, chunk: int = 100, reps: int = 3) -> dict:
    import torch

    N = w["natoms"]
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    # every host buffer the chunk touches is pinned, inputs and outputs alike
    pos, vel = pin(w["pos"]), pin(w["vel"])
    Z = pin(np.full(N, 18, dtype=np.int32))
    mass = pin(np.array(np.broadcast_to(np.asarray(w["mass"], dtype=np.float64), (N,))))
    out = tuple(pin(np.zeros((N, 3))) for _ in range(3))
    sim = make_sim(w, "mixed", device=device)
    sim.update_forces()
    sim.do_steps(chunk)  # warm: graph built
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        sim.set_atoms(pos, vel, Z=Z, mass=mass)
        sim.update_forces()
        sim.do_steps(chunk)
        log = sim.thermo_log()
        p, v, a = sim.atoms(out=out)
        times.append(time.perf_counter() - t0)
    t = min(times)
    h2d = N * (24 + 24 + 4 + 8)
    d2h = N * 72 + len(log) * 22 * 8
    return {"value": N * chunk / t, "unit": "atom-steps/s", "h2d_bytes_per_step": h2d / chunk,
            "d2h_bytes_per_step": d2h / chunk, "chunk_steps": chunk,
            "note": "per chunk: set_atoms from pinned host arrays, UpdateForces, 100 steps, thermo log and state read back into pinned host arrays"}


# Secondary, compute-side roofline of the LJ step: about 30 flops per pair evaluation and, with
# full lists, (4/3) pi (rc/sigma)^3 rho* pair evaluations inside the cutoff per atom-step; the
# peak is the nominal FP32 CUDA-core rate at the SM clock measured during the timed region.
LJ_FLOPS_PER_PAIR = 30
FP32_LANES_PER_SM = 128
NUM_SMS = 152


def flop_roofline(atom_steps_per_s: float, rho_star: float, clocks: dict) -> dict:
    pairs = 4.0 / 3.0 * math.pi * 2.5 ** 3 * rho_star
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    peak = NUM_SMS * FP32_LANES_PER_SM * 2 * mhz * 1e6 / 1e12
    achieved = atom_steps_per_s * pairs * LJ_FLOPS_PER_PAIR / 1e12
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "flops_per_pair": LJ_FLOPS_PER_PAIR, "pairs_per_atom_step": pairs,
            "peak_source": f"nominal FP32: {NUM_SMS} SMs x {FP32_LANES_PER_SM} lanes x 2 flop x {mhz:.0f} MHz"}


def profiled_traffic(name: str):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<name> (None if absent)."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return int(line.split(":", 1)[1])
    return None


def measure_drift(w, device: int, steps: int) -> dict:
    """NVE drift of the LJ liquid in both paths from the same melted state (nve_drift)."""
    return nve_drift(lambda prec: make_sim(w, prec, device=device), w["natoms"], w["dt"], steps)


def lj_batch_plugins(skin_sigma: float):
    from lpmd2_gb300 import gbmd

    rc = 2.5 * SIGMA
    dt = 0.005 * lj_tau()
    return (gbmd.Plugin("verletlist", f"cutoff {rc!r} skin {skin_sigma * SIGMA!r} maxneighbors 512"),
            gbmd.Plugin("lennardjones", f"sigma {SIGMA} epsilon {EPS} cutoff {rc!r}"),
            gbmd.Plugin("velocityverlet", f"dt {dt!r}"))


def lj_tau() -> float:
    from lpmd2_gb300 import inputs as I

    return I.lj_reduced_units(SIGMA, EPS, MASS)["tau_fs"]


def make_batch(systems, precision: str, device: int, params: dict):
    from lpmd2_gb300 import gbmd

    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems], device=device)
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    cm, pot, integ = lj_batch_plugins(params["skin_sigma"])
    b.set_cell_manager(cm)
    b.add_potential(pot)
    b.set_integrator(integ)
    b.set_precision(precision)
    b.set_option("graph_block", GRAPH_BLOCK)
    b.set_option("cell_scale", params["cell_scale"])
    b.set_option("lanes_per_atom", params.get("lanes_per_atom", 1))
    return b


def time_batch(b, device: int, warm: int, steps: int) -> float:
    """Device ms of `steps` steps in one call on the batch's stream (events around it), after
    `warm` untimed steps (at least one graph block, so the graph is captured before)."""
    import torch

    b.update_forces()
    b.do_steps(max(warm, GRAPH_BLOCK))
    st = torch.cuda.ExternalStream(b.stream, device=device)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.do_steps(steps)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1)


def batched_ensemble(device: int, steps: int, nsys: int = 512, rank: int = 0, world: int = 1, dist=None) -> dict:
    """The batched ensemble (512 LJ systems, N log-uniform in [256, 32000] as 4k^3, rho* in
    [0.70, 0.95], T* in [0.7, 2.0]): autotune on a sample, then time the whole batch in both
    precisions.  With several GPUs each rank takes its share of the systems (split by atom
    count, no exchange) and the slowest rank's time counts."""
    from lpmd2_gb300 import inputs as I
    from lpmd2_gb300.autotune import tune_batch
    from lpmd2_gb300.serve import partition

    everything = I.lj_ensemble(nsys, seed=4)
    total_atoms = sum(s["natoms"] for s in everything)
    mine = partition([s["natoms"] for s in everything], world)[rank]
    systems = [everything[k] for k in mine]
    natoms = sum(s["natoms"] for s in systems)
    t0 = time.perf_counter()
    sample = systems[:: max(1, nsys // 64)]
    best, trials = tune_batch(lambda p: make_batch(sample, "mixed", device, p),
                              lambda b: time_batch(b, device, 20, 40) / 40)
    tune_s = time.perf_counter() - t0
    b = make_batch(systems, "mixed", device, best)
    ms = time_batch(b, device, 20, steps)
    st = b.stats()
    b.close()
    k64 = max(GRAPH_BLOCK, steps // 5 // GRAPH_BLOCK * GRAPH_BLOCK)
    b64 = make_batch(systems, "fp64", device, best)
    ms64 = time_batch(b64, device, GRAPH_BLOCK, k64)
    b64.close()
    ms, ms64 = allmax(dist, ms), allmax(dist, ms64)
    value = total_atoms * steps / (ms * 1e-3)
    value64 = total_atoms * k64 / (ms64 * 1e-3)
    # the other end of the size range: 512 systems of the ensemble's smallest size (FCC 4^3,
    # 256 atoms), where launches per step and the rebuild chain weigh most against the work
    small = [I.lj_system(4, 0.70 + 0.25 * (q % 7) / 6, 0.7 + 1.3 * (q % 5) / 4, seed=900 + q) for q in range(nsys)]
    bs = make_batch(small, "mixed", device, dict(best, lanes_per_atom=1))
    ms_small = time_batch(bs, device, 20, steps)
    bs.close()
    small_atoms = sum(q["natoms"] for q in small)
    return {"workload": f"lj_ensemble_{nsys}", "seed": 4, "systems": nsys, "natoms_total": total_atoms,
            "systems_this_rank": len(systems), "natoms_this_rank": natoms,
            "natoms_min": min(s["natoms"] for s in everything), "natoms_max": max(s["natoms"] for s in everything),
            "steps": steps, "value": value, "unit": "atom-steps/s", "ms_per_step": ms / steps,
            "fp64_value": value64, "speedup_vs_fp64": value / value64, "tuned": best, "tuning_trials": trials,
            "tuning_s": tune_s, "device_bytes": st["device_bytes"],
            "small_systems": {"systems": nsys, "natoms_each": 256, "ms_per_step": ms_small / steps,
                              "value": small_atoms * steps / (ms_small * 1e-3)},
            "launch": "one launch per kernel for all systems; 10-step blocks as one CUDA graph"}


def served_stream(device: int, njobs: int, rate: float, rank: int = 0, world: int = 1, dist=None) -> dict:
    """Poisson job stream (70 % LJ, 30 % Sutton-Chen Cu; N log-uniform in [500, 200000];
    steps uniform in [1000, 20000]) through the job server with a 150 GB budget per GPU.
    With several GPUs every rank serves its share of the stream (split by atoms x steps)."""
    from lpmd2_gb300 import inputs as I
    from lpmd2_gb300.serve import GbmdBackend, Server, partition, summarize

    everything = I.job_stream(njobs, rate, seed=5)
    mine = partition([4 * j["k"] ** 3 * j["steps"] for j in everything], world)[rank]
    jobs = [everything[k] for k in mine]
    srv = Server(GbmdBackend(device=device), budget_bytes=150e9, max_batches=8, max_systems=512)
    barrier(dist)
    t0 = time.perf_counter()
    res = srv.serve(jobs, I.materialize_job)
    wall = time.perf_counter() - t0
    if dist is not None:
        gathered = [None] * world
        dist.all_gather_object(gathered, [(r.natoms, r.steps, r.arrival, r.finished, r.error) for r in res])
        from lpmd2_gb300.serve import JobResult

        res = [JobResult(0, "", n, st, a, finished=f, error=e) for part in gathered for (n, st, a, f, e) in part]
        wall = allmax(dist, wall)
    out = summarize(res, wall)
    work = {"lj": 0, "sc": 0}
    for j in everything:
        work[j["kind"]] += 4 * j["k"] ** 3 * j["steps"]
    out.update({"rate_jobs_per_s": rate, "seed": 5, "budget_bytes": 150e9, "batches": srv.batches_started,
                "peak_budget_used_bytes": srv.peak_used, "atom_steps_by_kind": work,
                "note": "latency = completion - arrival, wall clock; payloads generated before the clock starts"})
    return out


def sc_batched_rate(device: int, nsys: int = 48, steps: int = 40) -> dict:
    """The batched engine's rate on Sutton-Chen copper systems of the served stream's sizes (FCC
    k^3 cells, k of the stream's copper jobs), with the job server's plugins: the copper half of
    the reference the served throughput is compared with."""
    from lpmd2_gb300 import gbmd
    from lpmd2_gb300 import inputs as I
    from lpmd2_gb300.serve import GbmdBackend

    jobs = [j for j in I.job_stream(4 * nsys, 100.0, seed=5) if j["kind"] == "sc"][:nsys]
    systems = [I.materialize_job(j) for j in jobs]
    be = GbmdBackend(device=device)
    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems], device=device)
    for k, sy in enumerate(systems):
        b.set_atoms(k, sy["pos"], sy["vel"], Z=sy["Z"], mass=sy["mass"])
    cm, pot, integ = be.plugins("sc")
    b.set_cell_manager(cm)
    b.add_potential(pot)
    b.set_integrator(integ)
    b.set_precision("mixed")
    b.set_option("graph_block", GRAPH_BLOCK)
    ms = time_batch(b, device, 20, steps)
    b.close()
    natoms = sum(sy["natoms"] for sy in systems)
    return {"systems": nsys, "natoms": natoms, "steps": steps, "value": natoms * steps / (ms * 1e-3),
            "unit": "atom-steps/s"}


def budget_burst(device: int, njobs: int = 80, k: int = 80, steps: int = 50) -> dict:
    """A burst of large LJ jobs (FCC k^3 = 2,048,000 atoms each, rho* 0.8, T* 1.2, `steps` steps,
    all arriving at once) whose footprints add up to more than the 150 GB budget: the server
    admits as many as fit and the rest wait for memory.  Every job carries the same payload
    (made once, before the clock starts)."""
    from lpmd2_gb300 import inputs as I
    from lpmd2_gb300.serve import GbmdBackend, Server, summarize

    payload = I.lj_system(k, 0.8, 1.2, seed=51)
    jobs = [dict(id=q, kind="lj", k=k, steps=steps, arrival=0.0) for q in range(njobs)]
    srv = Server(GbmdBackend(device=device), budget_bytes=150e9, max_batches=8, max_systems=512)
    t0 = time.perf_counter()
    res = srv.serve(jobs, lambda j: payload)
    wall = time.perf_counter() - t0
    out = summarize(res, wall)
    out.update({"jobs_atoms_each": payload["natoms"], "steps_each": steps, "budget_bytes": 150e9,
                "peak_budget_used_bytes": srv.peak_used, "batches": srv.batches_started,
                "note": "all jobs arrive at t = 0; admission against the budget"})
    return out


def make_eam_sim(precision: str, device: int = 0, state: dict | None = None, ncell: int = 50):
    """Sutton-Chen copper, FCC ncell^3 at a = 3.61 A minus 1 % of the sites, 300 K (or `state`),
    linkedcell with cells of edge 2a = cutoff, velocityverlet dt 2 fs."""
    from lpmd2_gb300 import gbmd
    from lpmd2_gb300 import inputs as I

    w = I.sc_cu_system(ncell, seed=3)
    state = state or w
    c = I.SC_CU
    nx = int(round(w["L"][0] / (2 * c["a"])))
    sim = gbmd.Simulation(w["natoms"], w["L"], device=device)
    sim.set_atoms(state["pos"], state["vel"], Z=w["Z"], mass=w["mass"])
    sim.set_cell_manager(gbmd.Plugin("linkedcell", f"cutoff {2 * c['a']!r} nx {nx} ny {nx} nz {nx}"))
    sim.add_potential(gbmd.Plugin("suttonchen", f"e {c['e']} a {c['a']} n {c['n']} m {c['m']} c {c['c']} "
                                                f"cutoff {2 * c['a']!r}"))
    sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 2.0"))
    sim.set_precision(precision)
    sim.set_option("graph_block", GRAPH_BLOCK)
    return sim, w["natoms"]


def eam_metal(device: int, steps: int, drift_steps: int = 5000, ncell: int = 50) -> dict:
    """Sutton-Chen copper: FCC 50^3 at a = 3.61 A with 1 % of the sites removed (495,000 atoms),
    300 K, linkedcell nx 25 (cell edge = cutoff = 7.22 A), velocityverlet dt 2 fs.  Mixed and
    FP64 throughput; the mixed path's force RMS, energy and virial-pressure errors against FP64
    at the same positions, 20 steps from the lattice and after the timed run; and the NVE drift
    of both paths over `drift_steps` steps (5,000 x 2 fs = 10 ps) from the lattice."""
    from lpmd2_gb300 import inputs as I

    w = I.sc_cu_system(ncell, seed=3)
    N = w["natoms"]

    # the device's Verlet skin (linkedcell leaves it to the device), chosen by timing
    from lpmd2_gb300.autotune import tune_skin

    def with_skin(skin):
        sim = make_eam_sim("mixed", device, w, ncell)[0]
        sim.set_option("skin", skin)
        return sim

    skin, skin_trials = tune_skin(with_skin, lambda sim: time_batch(sim, device, 30, 150) / 150)

    def make(prec, state):
        sim = make_eam_sim(prec, device, state, ncell)[0]
        sim.set_option("skin", skin)
        return sim

    def errors(state) -> dict:
        sm, s64 = make("mixed", state), make("fp64", state)
        sm.update_forces()
        s64.update_forces()
        am, a64 = sm.atoms()[2], s64.atoms()[2]
        tm, t64 = sm.thermo(), s64.thermo()
        sm.close()
        s64.close()
        return {"force_rms_rel_err_vs_fp64": float(np.sqrt(np.sum((am - a64) ** 2) / np.sum(a64 ** 2))),
                "epot_rel_err_vs_fp64": abs(tm["potential_energy"] - t64["potential_energy"]) / abs(t64["potential_energy"]),
                "virial_pressure_rel_err_vs_fp64": abs(tm["virial_pressure"] - t64["virial_pressure"])
                / abs(t64["virial_pressure"]),
                "epot_ev": t64["potential_energy"], "virial_pressure_mpa": t64["virial_pressure"]}

    # the state 20 FP64 steps from the lattice (where the tests compare with the oracle)
    s20 = make("fp64", w)
    s20.update_forces()
    s20.do_steps(20)
    p20, v20, _ = s20.atoms()
    s20.close()
    err20 = errors(dict(w, pos=p20, vel=v20))
    # time the mixed path from the lattice; its final (thermalised) state is the second point
    # where the errors are measured (on the perfect lattice the forces nearly cancel)
    sm = make("mixed", w)
    ms = time_batch(sm, device, 20, steps)
    st = sm.stats()
    pos, vel, _ = sm.atoms()
    sm.close()
    err_hot = errors(dict(w, pos=pos, vel=vel))
    s64 = make("fp64", w)
    k64 = max(GRAPH_BLOCK, steps // 5 // GRAPH_BLOCK * GRAPH_BLOCK)
    ms64 = time_batch(s64, device, GRAPH_BLOCK, k64)
    s64.close()
    value, value64 = N * steps / (ms * 1e-3), N * k64 / (ms64 * 1e-3)
    out = {"workload": "sc_cu_fcc50_vac1pct", "seed": 3, "natoms": N, "steps": steps, "value": value,
           "unit": "atom-steps/s", "ms_per_step": ms / steps, "ns_per_day": value / N * 2.0 * 86400 * 1e-6,
           "fp64_value": value64, "speedup_vs_fp64": value / value64,
           "errors_20_fp64_steps": err20, "errors_after_timed_run": dict(err_hot, at=f"after {20 + steps} mixed steps"),
           "skin_a": skin, "skin_trials": skin_trials,
           "neighbor_mode": st["neighbor_mode"], "list_radius": st["list_radius"]}
    if drift_steps > 0:
        out["drift"] = nve_drift(lambda prec: make(prec, w), N, 2.0, drift_steps)
    return out


def nve_drift(make, natoms: int, dt_fs: float, steps: int, chunk: int = 1000) -> dict:
    """NVE total-energy drift of the mixed and the FP64 path: slope of a linear fit of the
    per-step total energy over `steps` steps, in eV/atom/ns, and the RMS fluctuation."""
    out = {"steps": steps, "ns": steps * dt_fs * 1e-6}
    for prec in ("mixed", "fp64"):
        s = make(prec)
        s.update_forces()
        s.thermo_log()
        logs = []
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            s.do_steps(k)
            logs.append(s.thermo_log())
            done += k
        s.close()
        log = np.concatenate(logs)
        t_ns = log[:, 0] * dt_fs * 1e-6
        out[f"{prec}_ev_per_atom_per_ns"] = float(np.polyfit(t_ns, log[:, 3], 1)[0]) / natoms
        out[f"{prec}_etot_rms_fluct_ev_per_atom"] = float(np.std(log[:, 3])) / natoms
    out["mixed_minus_fp64_ev_per_atom_per_ns"] = out["mixed_ev_per_atom_per_ns"] - out["fp64_ev_per_atom_per_ns"]
    return out


if __name__ == "__main__":
    main()
