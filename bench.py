"""Benchmark: atom-steps/s of the LJ velocity-Verlet step on one GB300.

Workload (the headline configuration): a single periodic LJ box of
1,000,000 atoms -- FCC, 50 x 50 x 100 unit cells at rho* = 0.8442, seeded
Maxwell-Boltzmann velocities at T* = 0.72 with zero momentum, r_cut = 2.5
sigma, skin 0.3 sigma, NVE velocity Verlet at dt* = 0.005.  One bench step is
one integrator step (kick, drift, wrap, neighbour-list check/rebuild, forces,
kick) over all atoms.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints one JSON line: `value` = mixed-path atom-steps/s with the state
resident in HBM (CUDA events on the engine's stream), `e2e` = the same metric
through the C ABI with host buffers (upload + K steps + download inside the
timed region), the plain FP64 GPU path beside it, force error against the
FP64 oracle on sampled rows, the force kernel's roofline, and the oracle's
CPU throughput on a bounded sample.  The reference arm (`--impl reference`)
times the reference algorithm's CPU restatement (the oracle: O(N^2)
all-pairs, all host threads) on bounded row samples of the same workload.
Multi-GPU runs are replicas: each rank integrates its own box (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s on 1 GB300, mixed/batched vs plain FP64; force err vs FP64 oracle"
K_B = 1.380648528
CELLS = (50, 50, 100)
RHO = 0.8442
T_STAR = 0.72
DT = 0.005
SKIN = 0.3
# algorithmic HBM bytes per atom of one force launch (mixed path, full list,
# no Newton-3): list 4 B x 77.6 candidates (4/3 pi 2.8^3 rho*), own mirror 16,
# count 4, force write 24, potential + temp write 16, velocity read+write 48.
LIST_CANDIDATES = 4.0 / 3.0 * np.pi * (2.5 + SKIN) ** 3 * RHO
BYTES_PER_ATOM_FORCE = 4.0 * LIST_CANDIDATES + 16 + 4 + 24 + 16 + 48


def workload_config(n_atoms):
    name = "lj_fcc_1M_nve" if tuple(CELLS) == (50, 50, 100) else f"lj_fcc_{n_atoms}_nve"
    return {"workload": name, "atoms": int(n_atoms),
            "lattice": f"FCC {CELLS[0]}x{CELLS[1]}x{CELLS[2]} unit cells", "rho_star": RHO,
            "t_star": T_STAR, "r_cut_sigma": 2.5, "skin_sigma": SKIN, "dt_star": DT,
            "ensemble": "NVE velocity Verlet", "seeded": True,
            "l2": "no flush: per-step inputs (neighbour list ~310 MB + state ~120 MB) exceed the 129 MB L2"}


def make_system(seed: int):
    from moldyn_gb300.initializer import UnitCell, lattice_positions, maxwell_boltzmann
    a = (4.0 / RHO) ** (1.0 / 3.0)
    pos = lattice_positions(UnitCell.FCC, CELLS, a)
    box = np.array(CELLS, dtype=np.float64) * a
    vel = maxwell_boltzmann(len(pos), T_STAR * 100.0 / K_B, 1.0, seed)
    return pos, vel, box


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.05)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = [ln.split(",") for ln in open(self.f.name).read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_atom():
    """DRAM bytes per atom of one mixed force launch from the committed ncu
    summary (profiles/force_mixed_traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "force_mixed_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["dram_bytes_per_atom"])
    return None


# ---------------------------------------------------------------------------
def oracle_rows_sample(pos, box, target_s: float, nthreads: int):
    """Time rows of the oracle's O(N^2) update_force (the reference algorithm)
    on the host cores; returns (rows, seconds, forces of those rows)."""
    from oracle import oracle as o
    n = len(pos)
    st = o.OracleState([n], pos, np.zeros_like(pos), [1.0], box, o.pot_table(1, default=(1.0, 1.0)))
    rows = max(nthreads * 4, 64)
    t0 = time.perf_counter()
    st.update_force(nthreads=nthreads, rows=(0, rows))
    dt = time.perf_counter() - t0
    rows = int(min(n, max(rows, rows * target_s / max(dt, 1e-6))))
    t0 = time.perf_counter()
    st.update_force(nthreads=nthreads, rows=(0, rows))
    dt = time.perf_counter() - t0
    return rows, dt, st.force[:rows].copy(), st.potential[:rows].copy()


def force_errors(f_gpu, f_ref):
    fmag = np.sqrt((f_ref ** 2).sum(axis=1))
    rms = float(np.sqrt((fmag ** 2).mean()))
    err = np.sqrt(((f_gpu - f_ref) ** 2).sum(axis=1))
    return {"max_rel": float((err / np.maximum(fmag, rms)).max()),
            "max_abs_over_rms": float(err.max() / rms),
            "rms_over_rms": float(np.sqrt((err ** 2).mean()) / rms),
            "definition": "per atom |dF_i| / max(|F_i|, rms|F|); rms |dF| / rms |F|"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    pos, vel, box = make_system(seed=1234)
    n = len(pos)
    from oracle import oracle as o
    st = o.OracleState([n], pos, vel, [1.0], box, o.pot_table(1, default=(1.0, 1.0)))
    # size one sampled step so the whole run ends within ~2 minutes
    per_step = min(0.5, 100.0 / max(args.steps + args.warmup, 1))
    rows, dt, _, _ = oracle_rows_sample(pos, box, per_step, nthreads)
    for _ in range(args.warmup):
        st.update_force(nthreads=nthreads, rows=(0, rows))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st.update_force(nthreads=nthreads, rows=(0, rows))
    t = time.perf_counter() - t0
    # one O(N^2) step over all N atoms costs (t/steps) * N/rows; atom-steps/s = rows / (t/steps)
    value = rows * args.steps / t
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps * n / rows,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded FCC lattice, rho*=0.8442, Maxwell-Boltzmann T*=0.72",
            "impl": "reference",
            "config": dict(workload_config(n), precision="fp64 (reference algorithm: all-pairs O(N^2))"),
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": nthreads, "kind": "port",
                             "sample": f"rows 0..{rows} of one all-pairs update_force per step "
                                       f"(extrapolated from {rows} of {n} rows)"},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from moldyn_gb300.engine import Engine

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    pos, vel, box = make_system(seed=1234 + rank)
    n = len(pos)
    types = np.zeros(n, dtype=np.uint16)

    # ---- mixed path, state resident in HBM --------------------------------
    eng = Engine(precision="mixed", skin=SKIN, profile=True, device=local)
    eng.set_potential(0, 0, 1.0, 1.0)
    eng.upload(types, pos, vel, [1.0], box)
    eng.compute_forces()
    eng.step(args.warmup, DT)
    eng.synchronize()
    eng.reset_stats()
    stream = torch.cuda.ExternalStream(eng.stream_ptr)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        eng.step(args.steps, DT)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier()
    t_ms = max_over_ranks(ev0.elapsed_time(ev1))
    st = eng.stats()
    clocks = clk.summary()
    value = world * n * args.steps / (t_ms * 1e-3)
    force_ms_avg = st.force_ms / max(st.force_launches, 1)
    # thermalised end state: positions and the forces the mixed path computed there
    end = eng.download()
    eng.close()

    if args.legs == "mixed":
        if rank == 0:
            print(json.dumps({"legs": "mixed", "value": value, "ms_per_step": t_ms / args.steps,
                              "force_kernel_ms": force_ms_avg, "threads_per_atom": st.threads_per_atom,
                              "rebuilds": st.rebuilds, "clocks": clocks}), flush=True)
        return

    # ---- end to end through the C ABI with host buffers -------------------
    eng = Engine(precision="mixed", skin=SKIN, threads_per_atom=st.threads_per_atom, device=local)
    eng.set_potential(0, 0, 1.0, 1.0)
    eng.upload(types, pos, vel, [1.0], box)       # warm the allocation path
    eng.compute_forces()
    eng.step(args.warmup, DT)
    eng.synchronize()
    barrier()
    t0 = time.perf_counter()
    eng.upload(types, pos, vel, [1.0], box)
    eng.compute_forces()
    eng.step(args.steps, DT)
    out = eng.download()
    t_e2e = max_over_ranks(time.perf_counter() - t0)
    e2e_launches = eng.stats().kernel_launches
    eng.close()
    h2d = n * (3 * 8 + 3 * 8 + 2 + 2 * 4)       # positions, velocities, types, (type, rank) staging
    d2h = n * (3 * 8 * 3 + 8 + 8)               # positions, velocities, forces, potential, temp
    e2e = {"value": world * n * args.steps / t_e2e, "unit": "atom-steps/s",
           "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
           "includes": "upload + initial forces + K steps + download, wall clock"}

    # ---- plain FP64 GPU path ---------------------------------------------
    k64 = max(3, min(args.steps, args.fp64_steps))
    eng = Engine(precision="fp64", skin=SKIN, device=local)
    eng.set_potential(0, 0, 1.0, 1.0)
    eng.upload(types, end["pos"], end["vel"], [1.0], box)
    eng.compute_forces()
    f_fp64_end = eng.download()["force"] if rank == 0 else None
    eng.step(3, DT)
    eng.synchronize()
    stream64 = torch.cuda.ExternalStream(eng.stream_ptr)
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    a0.record(stream64)
    eng.step(k64, DT)
    a1.record(stream64)
    a1.synchronize()
    t64 = max_over_ranks(a0.elapsed_time(a1))
    fp64_value = world * n * k64 / (t64 * 1e-3)
    fp64_tpa = eng.stats().threads_per_atom
    eng.close()

    if rank != 0:
        return

    # ---- CPU baseline (the oracle on a bounded sample) + force error ------
    nthreads = os.cpu_count() or 1
    # the oracle's rows at the thermalised end state of the timed run (a
    # perfect lattice has zero net forces, useless for an error measure)
    rows, tcpu, f_ref, _ = oracle_rows_sample(end["pos"], box, args.cpu_seconds, nthreads)
    cpu_value = rows / tcpu
    err_mixed = force_errors(end["force"][:rows], f_ref)
    err_fp64 = force_errors(f_fp64_end[:rows], f_ref)

    peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_ATOM_FORCE * n / (force_ms_avg * 1e-3) / 1e9
    tpa_traffic = ncu_traffic_per_atom()
    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair maths / i64 fixed-point force sums / f64 drift+reductions",
        "data": "synthetic: seeded FCC lattice, rho*=0.8442, Maxwell-Boltzmann T*=0.72, zero momentum",
        "config": dict(workload_config(n), precision="mixed", threads_per_atom=st.threads_per_atom,
                       neighbor_capacity=st.neighbor_capacity, rebuilds_in_timed_region=st.rebuilds,
                       parallelism="replicas" if world > 1 else "single GPU",
                       fp64_plain_path={"value": fp64_value, "unit": "atom-steps/s", "steps": k64,
                                        "threads_per_atom": fp64_tpa},
                       mixed_over_fp64=value / fp64_value,
                       force_err_vs_fp64_oracle={"mixed": err_mixed, "fp64_plain": err_fp64,
                                                 "atoms_sampled": rows,
                                                 "state": "end of the timed run (thermalised)"},
                       force_kernel_ms=force_ms_avg, integrate_kernel_ms=st.integrate_ms / max(
                           st.integrate_launches, 1)),
        "e2e": e2e,
        "gpu_launches": st.kernel_launches,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": "k_force_mixed", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "bytes_per_atom": BYTES_PER_ATOM_FORCE, "avg_launch_ms": force_ms_avg,
                     "traffic": (tpa_traffic * n if tpa_traffic else None)},
        "cpu_baseline": {"value": cpu_value, "unit": "atom-steps/s", "cores": nthreads, "kind": "port",
                         "sample": f"oracle all-pairs update_force, rows 0..{rows} of {n} "
                                   f"(extrapolated from {rows} rows)"},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--cells", default="50,50,100",
                    help="FCC unit cells (profiling uses smaller boxes; the bench line uses the default)")
    ap.add_argument("--legs", default="all", choices=["all", "mixed"],
                    help="'mixed' runs only the timed mixed leg (for profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    global CELLS
    CELLS = tuple(int(c) for c in args.cells.split(","))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
