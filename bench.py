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


def cpu_sample(seconds_target: float = 15.0, procs: int | None = None) -> dict:
    """Times the reference CPU algorithm (oracle/_ref where built, else the C restatement) on
    a bounded sample: a 4,000-atom cut of the same liquid (FCC 10^3 at rho* 0.8442, T* 1.5,
    same cutoff), linkedcell + velocityverlet, one replica per host core."""
    import multiprocessing as mp

    ncores = procs or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(ncores) as pool:
        res = pool.map(_cpu_worker, [seconds_target / 3.0] * ncores)
    steps = sum(r[0] for r in res)
    atoms = res[0][1]
    wall = max(r[2] for r in res)
    kind = res[0][3]
    return {"value": steps * atoms / wall, "unit": "atom-steps/s", "cores": ncores, "kind": kind,
            "sample": f"{ncores} replicas x {steps // ncores} steps of a {atoms}-atom cut of the liquid "
                      f"(FCC 10^3, linkedcell nx 4, velocityverlet, 2 force evaluations per step as the "
                      f"reference does), {wall:.1f} s"}


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
    one = time.perf_counter() - t0
    k = max(2, int(budget / max(one, 1e-3)))
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
    cb = cpu_sample(seconds_target=float(os.environ.get("GBMD_CPU_SECONDS", "20")))
    out = {
        "metric": "atom-steps/s", "value": cb["value"], "unit": "atom-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * w["natoms"] / cb["value"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": "lj_liquid_fcc40_256k", "natoms": w["natoms"], "precision": "fp64",
                   "sampled_as": cb["sample"]},
        "cpu_baseline": {"value": cb["value"], "unit": cb["unit"], "cores": cb["cores"], "kind": cb["kind"],
                         "sample": cb["sample"]},
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
    ap.add_argument("--melt", type=int, default=1000, help="untimed mixed steps that melt the lattice")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--profile", action="store_true",
                    help="short direct-launch run of the workload for ncu (no timing, no JSON)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"], help="with --profile")
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
    sim = make_sim(w, "mixed", device=local)
    sim.update_forces()
    if args.melt:
        sim.do_steps(args.melt)
    p_melt, v_melt, _ = sim.atoms()
    w_melt = dict(w, pos=p_melt, vel=v_melt)
    sim.do_steps(args.warmup)
    sim.synchronize()

    stream = torch.cuda.ExternalStream(sim.stream, device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def timed_blocks(s, k_total):
        """k_total steps in graph blocks; L2 flushed (256 MB write) before every block,
        outside the timed events.  Returns summed device time in ms."""
        st = torch.cuda.ExternalStream(s.stream, device=local)
        ms = 0.0
        done = 0
        while done < k_total:
            b = min(GRAPH_BLOCK, k_total - done)
            with torch.cuda.stream(st):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            s.do_steps(b)
            e1.record(st)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            done += b
        return ms

    stats0 = sim.stats()
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = timed_blocks(sim, args.steps)
    torch.cuda.synchronize()
    barrier(dist)
    stats1 = sim.stats()
    ms = allmax(dist, ms)
    value = N * args.steps * world / (ms * 1e-3)
    th_log = sim.thermo_log()

    # plain FP64 GPU path on the same (melted) state
    sim64 = make_sim(w_melt, "fp64", device=local)
    sim64.update_forces()
    k64 = max(GRAPH_BLOCK, (args.steps // 5) // GRAPH_BLOCK * GRAPH_BLOCK)
    sim64.do_steps(GRAPH_BLOCK)
    ms64 = timed_blocks(sim64, k64)
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
    del simm, sim64b

    # kernel timing pass (direct launches, events around the force kernel on its stream)
    kt = kernel_times(w_melt, local)

    # end to end through the public API with pinned host buffers: upload the state, run a
    # 100-step chunk, read back the per-step thermo and the final state
    e2e = end_to_end(w_melt, local)

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_kind = "measured" if "hbm_gbs" in peaks else "fallback"
    force_bytes_per_atom = 120.0  # own position 24 + v, a_old 48 in; v, a 48 out
    achieved = force_bytes_per_atom * N / (kt["force_ms"] * 1e-3) / 1e9 if kt["force_ms"] else None
    step_bytes_per_atom = 168.0
    step_achieved = step_bytes_per_atom * N * args.steps / (ms * 1e-3) / 1e9

    # energy drift over the timed region (linear fit of the total energy)
    drift = None
    if len(th_log) > 2:
        t_ps = th_log[:, 0] * w["dt"] * 1e-3
        slope = np.polyfit(t_ps, th_log[:, 3], 1)[0]  # eV per ps
        drift = float(slope * 1e3 / N)  # eV/atom/ns

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        cpu = cpu_sample(seconds_target=float(os.environ.get("GBMD_CPU_SECONDS", "15")))
    launches = stats1["kernel_launches"] - stats0["kernel_launches"]
    out = {
        "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64 (f64 integrate)",
        "data": "synthetic",
        "config": {"workload": "lj_liquid_fcc40_256k", "natoms": N, "rho_star": RHO_STAR, "T_star": T_STAR,
                   "cutoff_sigma": 2.5, "skin_sigma": 0.3, "dt_fs": w["dt"], "precision": "mixed",
                   "graph_block": GRAPH_BLOCK, "melt_steps": args.melt,
                   "l2": "flushed (256 MB write) before every 10-step graph block, outside the timing",
                   "parallelism": f"replicas x{world}"},
        "ns_per_day": value / N / world * w["dt"] * 86400 * 1e-6,
        "fp64_value": value64 * world, "fp64_ms_per_step": ms64 / k64, "speedup_vs_fp64": value / (value64 * world),
        "force_rms_rel_err_vs_fp64": frel, "epot_rel_err_vs_fp64": abs(e_m - e_64) / abs(e_64),
        "drift_ev_per_atom_per_ns": drift,
        "list_rebuilds_timed": stats1["list_rebuilds"] - stats0["list_rebuilds"],
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "traffic": None,
                     "kernel": "k_force32<pair> (fused LJ force + velocity kick)",
                     "bytes_per_atom": force_bytes_per_atom, "launch_ms": kt["force_ms"],
                     "peak_source": peak_kind},
        "step_roofline": {"achieved": step_achieved, "peak": peak, "unit": "GB/s", "frac": step_achieved / peak,
                          "bytes_per_atom_step": step_bytes_per_atom},
        "kernel_ms": kt,
        "e2e": e2e,
        "clocks": clk.summary(),
    }
    if cpu:
        out["cpu_baseline"] = cpu
    print(json.dumps(out))


def run_profile(args):
    """The workload with direct launches only (graph_mode 0), for ncu: melt, warm up, then
    --steps steps.  Every kernel of a step is a separate launch on the simulation's stream."""
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
    pos, vel = pin(w["pos"]), pin(w["vel"])
    sim = make_sim(w, "mixed", device=device)
    sim.update_forces()
    sim.do_steps(chunk)  # warm: graph built
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        sim.set_atoms(pos, vel, Z=18, mass=w["mass"])
        sim.update_forces()
        sim.do_steps(chunk)
        log = sim.thermo_log()
        p, v, a = sim.atoms()
        times.append(time.perf_counter() - t0)
    t = min(times)
    h2d = N * (24 + 24 + 4 + 8)
    d2h = N * 72 + len(log) * 22 * 8
    return {"value": N * chunk / t, "unit": "atom-steps/s", "h2d_bytes_per_step": h2d / chunk,
            "d2h_bytes_per_step": d2h / chunk, "chunk_steps": chunk,
            "note": "per chunk: set_atoms from pinned host arrays, UpdateForces, 100 steps, thermo log and state read back"}


if __name__ == "__main__":
    main()
