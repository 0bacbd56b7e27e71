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
LIST_KW = {}   # --direct-list: {"direct_list": True}
# algorithmic HBM bytes per atom of one force launch (mixed path, full list,
# no Newton-3): list 4 B x 77.6 candidates (4/3 pi 2.8^3 rho*), own mirror 16,
# count 4, force write 24, potential + temp write 16, velocity read+write 48.
LIST_CANDIDATES = 4.0 / 3.0 * np.pi * (2.5 + SKIN) ** 3 * RHO
BYTES_PER_ATOM_FORCE = 4.0 * LIST_CANDIDATES + 16 + 4 + 24 + 16 + 48
# NVE chunks fuse the next step's kick + drift into the force launch: position
# read + write 64, frozen cell 4, rebuild mirror 16, mirror write 16.
BYTES_PER_ATOM_DRIFT = 64 + 4 + 16 + 16
# ... and those fused launches store neither the forces nor potential + temp
# (the chunk's last launch does)
BYTES_PER_ATOM_FUSED_SKIP = 24 + 16
ENGINE_CHUNK = 64   # steps per chunk of an eager Engine.step (no graph)


def fused_fraction(steps: int, chunk: int = ENGINE_CHUNK) -> float:
    """Share of the force launches of `steps` NVE steps that carry the fused
    drift: a chunk of n steps fuses (n - 1) rounded down to even."""
    fused, left = 0, steps
    while left > 0:
        n = min(chunk, left)
        fused += (n - 1) & ~1
        left -= n
    return fused / max(steps, 1)


DATA = "synthetic: seeded FCC lattice, rho*=0.8442, Maxwell-Boltzmann T*=0.72, zero momentum"


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


def make_positions_oracle():
    """The same FCC sites as make_system, from the oracle's restatement of
    initialize_particles_position (the reference arm loads no product code;
    update_force reads positions only)."""
    from oracle import oracle as o
    a = (4.0 / RHO) ** (1.0 / 3.0)
    pos = o.lattice("FCC", *CELLS, a)
    box = np.array(CELLS, dtype=np.float64) * a
    return pos, box


def issue_roofline(n_atoms, launch_ms, clocks):
    """The force kernel against the SMs' instruction issue rate (what bounds
    it; HBM does not): warp instructions per atom of one fused launch (ncu,
    committed) x atoms / launch time, against 4 schedulers x SMs x clock."""
    p = os.path.join(ROOT, "profiles", "force_mixed_traffic.json")
    if not os.path.exists(p) or not launch_ms:
        return None
    with open(p) as f:
        d = json.load(f)
    per_atom = d.get("warp_instructions_per_atom")
    if not per_atom:
        return None
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    achieved = per_atom * n_atoms / (launch_ms * 1e-3)
    peak = 4.0 * sms * mhz * 1e6
    return {"achieved": achieved, "peak": peak, "unit": "warp instructions/s", "frac": achieved / peak,
            "warp_instructions_per_atom": per_atom, "sm_mhz": mhz}


def fp64_pipe_fraction(atom_steps_per_s):
    """The plain FP64 path against GB300's FP64 pipe: FP64 instructions per
    atom-step (ncu, committed) x throughput / the measured DFMA rate."""
    r = fp64_rates()
    if not r:
        return {}
    achieved = r["fp64_pipe_thread_inst_per_atom_step"] * atom_steps_per_s
    return {"fp64_pipe": {"bound": "fp64 pipe", "achieved_inst_per_s": achieved, "peak_dfma_per_s": r["dfma_per_s"],
                          "frac": achieved / r["dfma_per_s"], "source": r["source"]}}


def timing_note(st, steps):
    """How the timed steps ran, from the engine's own counters."""
    if st.graph_launches:
        return (f"{st.graph_launches} CUDA-graph replays covering {steps} steps "
                f"({st.kernel_launches} kernel launches), graphs captured before the timed region")
    return f"eager launches ({st.kernel_launches} kernel launches)"


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


def fp64_rates():
    """FP64-pipe instructions per atom-step of the plain path's force pass and
    the measured DFMA rate (profiles/fp64_rates.json), or None."""
    p = os.path.join(ROOT, "profiles", "fp64_rates.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


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
    """The reference algorithm (the oracle's restatement of update_force: an
    O(N^2) all-pairs FP64 loop, parallel over rows like the reference's
    rayon loop) on all host threads.  One bench step is one sampled step: a
    contiguous range of rows of the full all-pairs step, sized so the whole
    run takes about a minute; the throughput is rows computed per second."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as o
    nthreads = os.cpu_count() or 1
    pos, box = make_positions_oracle()
    n = len(pos)
    st = o.OracleState([n], pos, np.zeros_like(pos), [1.0], box, o.pot_table(1, default=(1.0, 1.0)))
    per_step = min(1.0, max(0.05, 60.0 / max(args.steps + args.warmup, 1)))
    probe = 16 * nthreads
    t0 = time.perf_counter()
    st.update_force(nthreads=nthreads, rows=(0, probe))
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    rows = int(min(n, max(probe, rate * per_step)))
    for _ in range(args.warmup):
        st.update_force(nthreads=nthreads, rows=(0, rows))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st.update_force(nthreads=nthreads, rows=(0, rows))
    t = time.perf_counter() - t0
    value = rows * args.steps / t
    ms_step = 1e3 * t / args.steps
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA, "impl": "reference", "config": workload_config(n),
            "sampled_step": {"rows": rows, "of_rows": n, "ms": ms_step,
                             "full_step_ms_extrapolated": ms_step * n / rows,
                             "note": "a bench step of this arm is rows 0..rows of the all-pairs update_force"},
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": nthreads, "kind": "port",
                             "sample": f"rows 0..{rows} of the {n}-atom all-pairs update_force per step "
                                       f"(oracle restatement, {nthreads} threads)"},
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
    # the headline leg is the mixed path; --legs mixed --precision fp64 times
    # the plain FP64 path the same way (profiler captures)
    leg_precision = args.precision if args.legs == "mixed" else "mixed"

    def timed_leg(**kw):
        """K steps from the seeded start after W warm-up steps: device time
        (CUDA events on the engine's stream, max over ranks), stats, clocks,
        end state."""
        eng = Engine(precision=leg_precision, skin=SKIN, device=local, **LIST_KW, **kw)
        eng.set_potential(0, 0, 1.0, 1.0)
        eng.upload(types, pos, vel, [1.0], box)
        eng.compute_forces()
        eng.step(args.warmup, DT)
        eng.prepare_step(args.steps, DT)     # graph capture (runs nothing) before the timed region
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
        t = max_over_ranks(ev0.elapsed_time(ev1))
        st_ = eng.stats()
        end_ = eng.download()
        eng.close()
        return t, st_, clk.summary(), end_

    # per-launch events (force kernel time for the roofline); eager launches
    t_prof, st, clocks_prof, end = timed_leg(profile=True, threads_per_atom=args.tpa)
    force_ms_avg = st.force_ms / max(st.force_launches, 1)
    # the engine's fastest mode: chunks of GRAPH_STEPS steps replayed as one CUDA graph
    if args.graph_steps > 1:
        t_ms, st_g, clocks, _ = timed_leg(graph_steps=args.graph_steps, threads_per_atom=st.threads_per_atom)
    else:
        t_ms, st_g, clocks = t_prof, st, clocks_prof
    value = world * n * args.steps / (t_ms * 1e-3)

    if args.legs == "mixed":
        phases = None
        if args.trace:
            te = Engine(precision="mixed", skin=SKIN, trace=True, device=local,
                        threads_per_atom=st.threads_per_atom, **LIST_KW)
            te.set_potential(0, 0, 1.0, 1.0)
            te.upload(types, end["pos"], end["vel"], [1.0], box)
            te.compute_forces()
            te.trace_phases()
            te.step(args.steps, DT)
            phases = te.trace_phases()
            te.close()
        if rank == 0:
            print(json.dumps({"legs": "mixed", "precision": leg_precision, "value": value,
                              "ms_per_step": t_ms / args.steps,
                              "eager_profiled_ms_per_step": t_prof / args.steps,
                              "force_kernel_ms": force_ms_avg, "threads_per_atom": st.threads_per_atom,
                              "rebuilds": st.rebuilds, "clocks": clocks, "k_pre_phases_us": phases}), flush=True)
        return

    # ---- end to end through the C ABI with host buffers -------------------
    # upload (host arrays -> device) + initial forces + K steps + download of
    # the whole state into host arrays, wall clock.  Warm-up: the same calls
    # once (the second upload of an unchanged shape keeps the device
    # allocations and the captured graphs, as a user's loop would).
    eng = Engine(precision="mixed", skin=SKIN, threads_per_atom=st.threads_per_atom, device=local,
                 graph_steps=max(args.graph_steps, 0), **LIST_KW)
    eng.set_potential(0, 0, 1.0, 1.0)
    host_out = {}
    eng.upload(types, pos, vel, [1.0], box)
    eng.compute_forces()
    eng.step(args.warmup, DT)
    eng.prepare_step(args.steps, DT)
    eng.download(host_out)
    eng.synchronize()
    eng.reset_stats()
    barrier()
    t0 = time.perf_counter()
    eng.upload(types, pos, vel, [1.0], box)
    eng.compute_forces()
    eng.step(args.steps, DT)
    out = eng.download(host_out)
    t_e2e = max_over_ranks(time.perf_counter() - t0)
    st_e2e = eng.stats()
    # the reference's solve loop with --frames-per-save 1: one step, then the
    # whole state back to the host, every step
    kf = max(3, min(args.steps, 50))
    eng.prepare_step(1, DT)
    eng.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(kf):
        eng.step(1, DT)
        eng.download(host_out)
    t_frames = max_over_ranks(time.perf_counter() - t0)
    eng.close()
    h2d = n * (3 * 8 + 3 * 8 + 2)               # positions, velocities, type ids
    d2h = n * (3 * 8 * 3 + 8 + 8)               # positions, velocities, forces, potential, temp
    e2e = {"value": world * n * args.steps / t_e2e, "unit": "atom-steps/s",
           "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
           "includes": ("upload of host arrays + initial forces + K steps + download of the whole state "
                        "into host arrays, wall clock; the copies go straight between the caller's "
                        "(pageable) arrays and device memory"),
           "graph_launches": st_e2e.graph_launches, "kernel_launches": st_e2e.kernel_launches,
           "every_step_download": {"value": world * n * kf / t_frames, "unit": "atom-steps/s", "steps": kf,
                                   "d2h_bytes_per_step": d2h,
                                   "includes": "per step: one step, then the full state to host buffers"}}

    # ---- plain FP64 GPU path ---------------------------------------------
    k64 = max(3, min(args.steps, args.fp64_steps or 50))
    eng = Engine(precision="fp64", skin=SKIN, device=local)
    eng.set_potential(0, 0, 1.0, 1.0)
    eng.upload(types, end["pos"], end["vel"], [1.0], box)
    eng.compute_forces()
    f_fp64_end = eng.download()["force"] if rank == 0 else None
    mac_fp64 = eng.macro(0)
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

    # the mixed path's macro parameters at the same state (its own forces,
    # potential and virial) against the FP64 path's
    em = Engine(precision="mixed", skin=SKIN, device=local)
    em.set_potential(0, 0, 1.0, 1.0)
    em.upload(types, end["pos"], end["vel"], [1.0], box)
    em.compute_forces()
    mac_mixed = em.macro(0)
    em.close()
    macro_err = {k: abs(mac_mixed[k] - mac_fp64[k]) / abs(mac_fp64[k])
                 for k in ("kinetic_energy", "potential_energy", "thermal_energy", "temperature", "pressure")}
    e_tot = mac_fp64["kinetic_energy"] + mac_fp64["potential_energy"]
    macro_err["total_energy"] = abs(mac_mixed["kinetic_energy"] + mac_mixed["potential_energy"] - e_tot) / abs(e_tot)
    macro_err["definition"] = ("|mixed - fp64| / |fp64| at the end state of the timed run; the FP64 GPU path "
                               "matches the oracle to ~1e-15 in the parity tests")

    # ---- CPU baseline (the oracle on a bounded sample) + force error ------
    nthreads = os.cpu_count() or 1
    # the oracle's rows at the thermalised end state of the timed run (a
    # perfect lattice has zero net forces, useless for an error measure)
    rows, tcpu, f_ref, _ = oracle_rows_sample(end["pos"], box, args.cpu_seconds, nthreads)
    cpu_value = rows / tcpu
    err_mixed = force_errors(end["force"][:rows], f_ref)
    err_fp64 = force_errors(f_fp64_end[:rows], f_ref)

    peak, peak_kind = measured_peaks()
    bytes_per_atom = BYTES_PER_ATOM_FORCE + fused_fraction(args.steps) * (BYTES_PER_ATOM_DRIFT -
                                                                          BYTES_PER_ATOM_FUSED_SKIP)
    achieved = bytes_per_atom * n / (force_ms_avg * 1e-3) / 1e9
    tpa_traffic = ncu_traffic_per_atom()
    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair maths / i64 fixed-point force sums / f64 drift+reductions",
        "data": DATA,
        "config": workload_config(n),
        "details": dict(precision="mixed", threads_per_atom=st.threads_per_atom,
                       neighbor_capacity=st.neighbor_capacity, rebuilds_in_timed_region=st_g.rebuilds,
                       timing=timing_note(st_g, args.steps),
                       eager_profiled={"value": world * n * args.steps / (t_prof * 1e-3),
                                       "ms_per_step": t_prof / args.steps,
                                       "note": "per-launch CUDA events; gives the force-kernel time of the roofline"},
                       parallelism="replicas" if world > 1 else "single GPU",
                       fp64_plain_path=dict({"value": fp64_value, "unit": "atom-steps/s", "steps": k64,
                                             "threads_per_atom": fp64_tpa}, **fp64_pipe_fraction(fp64_value)),
                       mixed_over_fp64=value / fp64_value,
                       macro_err_vs_fp64=macro_err,
                       force_err_vs_fp64_oracle={"mixed": err_mixed, "fp64_plain": err_fp64,
                                                 "atoms_sampled": rows,
                                                 "state": "end of the timed run (thermalised)"},
                       force_kernel_ms=force_ms_avg, integrate_kernel_ms=st.integrate_ms / max(
                           st.integrate_launches, 1)),
        "e2e": e2e,
        "gpu_launches": st_g.kernel_launches,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": "k_force_mixed", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "bytes_per_atom": bytes_per_atom, "fused_drift_share": fused_fraction(args.steps),
                     "avg_launch_ms": force_ms_avg,
                     "traffic": (tpa_traffic * n if tpa_traffic else None),
                     "issue": issue_roofline(n, force_ms_avg, clocks)},
        "cpu_baseline": {"value": cpu_value, "unit": "atom-steps/s", "cores": nthreads, "kind": "port",
                         "sample": f"oracle all-pairs update_force, rows 0..{rows} of {n} "
                                   f"(extrapolated from {rows} rows)"},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Other configurations (each prints its own JSON line; the default line is lj1m)

def _timed_steps(eng, nsteps, dt, **kw):
    """K steps on the engine's stream, CUDA-event timed; returns ms."""
    import torch
    stream = torch.cuda.ExternalStream(eng.stream_ptr)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    if kw.get("ensemble"):
        eng.ensemble_step(nsteps, dt)
    else:
        eng.step(nsteps, dt, **{k: v for k, v in kw.items() if k != "ensemble"})
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b)


def run_argon(args):
    """Argon, 1000 atoms on a 10^3 simple-cubic lattice (edge 3.338339 nm,
    m = 66.335, sigma = 0.3405 nm, eps/kB = 119.8 K), Maxwell-Boltzmann at
    273.15 K, Berendsen thermostat tau 10 -> 300 K and barostat (1, 5) ->
    1.01325, dt 0.002, 1000 steps: the reference's own units."""
    from moldyn_gb300.engine import Engine
    from moldyn_gb300.initializer import Barostat, Thermostat, UnitCell, lattice_positions, maxwell_boltzmann
    a, m, sig, eps = 3.338339, 66.335, 0.3405, 119.8 * K_B * 0.01
    pos = lattice_positions(UnitCell.U, (10, 10, 10), a)
    vel = maxwell_boltzmann(1000, 273.15, m, 7)
    box = np.full(3, 10 * a)
    n, steps = len(pos), args.steps
    res = {}
    for prec, ref in (("fp64", True), ("mixed", False)):
        e = Engine(precision=prec, reference_order=ref)
        e.set_potential(0, 0, sig, eps)
        e.upload(np.zeros(n, dtype=np.uint16), pos, vel, [m], box)
        e.compute_forces()
        th, ba = Thermostat.Berendsen(10.0), Barostat.Berendsen(1.0, 5.0)
        ms = _timed_steps(e, steps, 0.002, thermostat=th, target_temperature=300.0, barostat=ba,
                          target_pressure=1.01325)
        out = e.download()
        mac = e.macro(0)
        res[prec] = dict(value=n * steps / (ms * 1e-3), ms=ms, out=out, mac=mac, lam=th.lambda_, myu=ba.myu)
        e.close()
    # the oracle (reference algorithm) on the same trajectory, timed on the host
    from oracle import oracle as o
    st = o.OracleState([n], pos, vel, [m], box, o.pot_table(1, default=(sig, eps)))
    st.update_force(nthreads=os.cpu_count() or 1)
    oth, oba = o.Thermostat(o.BERENDSEN, 10.0, 0.0, 0.0), o.Barostat(1.0, 5.0, 0.0)
    t0 = time.perf_counter()
    st.step(0.002, nsteps=steps, barostat=oba, P0=1.01325, thermostat=oth, T0=300.0,
            nthreads=os.cpu_count() or 1)
    tcpu = time.perf_counter() - t0
    f64 = res["fp64"]["out"]
    d = f64["pos"] - st.pos
    d -= st.box * np.round(d / st.box)
    line = {"metric": METRIC, "value": res["mixed"]["value"], "unit": "atom-steps/s", "n_gpus": 1,
            "steps": steps, "higher_is_better": True, "dtype": "f32/i64-fixed/f64",
            "data": "synthetic: argon U lattice 10^3, seeded Maxwell-Boltzmann 273.15 K",
            "config": {"workload": "argon_1000_berendsen_TP", "atoms": n, "sigma_nm": sig, "eps": eps,
                       "mass": m, "dt_ps": 0.002, "thermostat": "Berendsen tau 10 -> 300 K",
                       "barostat": "Berendsen (1, 5) -> 1.01325",
                       "fp64_reference_order": {"value": res["fp64"]["value"],
                                                "max_pos_diff_vs_oracle_nm": float(np.abs(d).max()),
                                                "box_rel_diff_vs_oracle": float(np.abs(f64["box"] / st.box - 1).max()),
                                                "lambda": res["fp64"]["lam"], "oracle_lambda": oth.lambda_,
                                                "myu": res["fp64"]["myu"], "oracle_myu": oba.myu},
                       "final_T_K": res["mixed"]["mac"]["temperature"], "final_P": res["mixed"]["mac"]["pressure"],
                       "oracle_final_T_K": st.temperature(0), "oracle_final_P": st.pressure(0)},
            "cpu_baseline": {"value": n * steps / tcpu, "unit": "atom-steps/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": f"full run: {steps} steps of the oracle"}}
    print(json.dumps(line), flush=True)


def run_lj8m(args):
    """8,000,000 atoms: FCC 100x100x200 cells at rho* 0.8442, T* 0.72, Berendsen
    thermostat tau* 0.5 -> T* 0.72 and barostat (beta 1, tau_P* 5) -> P* 1.0,
    500 steps; per-kernel roofline.  The timed leg records per-launch events
    (force launches; step kernel + list-build kernel); a second run of the
    same steps with the step kernel's phase trace splits the step kernel from
    the list build."""
    global CELLS
    if not args.cells:
        CELLS = (100, 100, 200)
    from moldyn_gb300.engine import Engine
    from moldyn_gb300.initializer import Barostat, Thermostat
    pos, vel, box = make_system(seed=88)
    n = len(pos)
    T0 = T_STAR * 100.0 / K_B

    def leg(trace):
        e = Engine(precision="mixed", skin=SKIN, profile=not trace, trace=trace)
        e.set_potential(0, 0, 1.0, 1.0)
        e.upload(np.zeros(n, dtype=np.uint16), pos, vel, [1.0], box)
        e.compute_forces()
        th, ba = Thermostat.Berendsen(0.5), Barostat.Berendsen(1.0, 5.0)
        kw = dict(thermostat=th, target_temperature=T0, barostat=ba, target_pressure=1.0)
        e.step(args.warmup, DT, **kw)
        e.reset_stats()
        if trace:
            e.trace_phases()
        with ClockSampler(0) as clk:
            ms = _timed_steps(e, args.steps, DT, **kw)
        st = e.stats()
        phases = e.trace_phases() if trace else None
        mac = e.macro(0)
        end = e.download()
        e.close()
        return ms, st, phases, mac, end, clk.summary()

    ms, st, _, mac, end, clocks = leg(False)
    _, st_t, phases, _, _, _ = leg(True)
    peak, kind = measured_peaks()
    f_ms = st.force_ms / max(st.force_launches, 1)
    p_ms = st.integrate_ms / max(st.integrate_launches, 1)
    # the step kernel alone (its phases), per step; the list build per rebuild
    steps_t = max(phases["launches"], 1.0)
    pre_us = sum(v for k, v in phases.items() if k not in ("verlet_list", "launches", "rebuild_launches"))
    list_us = phases["verlet_list"]
    # k_pre algorithmic bytes per atom without a rebuild: pos r/w 64, vel r/w 48,
    # force read 24, cell 4, mirror write 16, mirror0 read 16, plus the coupled
    # steps' reduction pass over velocities, temp and potential (48)
    pre_bytes = 64 + 48 + 24 + 4 + 16 + 16 + 48
    pre_ms = pre_us / steps_t * 1e-3
    line = {"metric": METRIC, "value": n * args.steps / (ms * 1e-3), "unit": "atom-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "dtype": "f32/i64-fixed/f64", "data": "synthetic: FCC 100x100x200, seeded T*=0.72",
            "config": {"workload": "lj_fcc_8M_berendsen_TP" if n == 8000000 else f"lj_fcc_{n}_berendsen_TP",
                       "atoms": n, "rebuilds": st.rebuilds,
                       "threads_per_atom": st.threads_per_atom, "final_T_star": mac["temperature"] * K_B / 100.0,
                       "final_P_star": mac["pressure"], "final_box": end["box"].tolist()},
            "clocks": clocks,
            "kernels": {"k_force_mixed": {"avg_ms": f_ms, "bytes_per_atom": BYTES_PER_ATOM_FORCE,
                                          "achieved_GBps": (BYTES_PER_ATOM_FORCE * n / (f_ms * 1e-3) / 1e9
                                                            if f_ms > 0 else None),
                                          "peak_GBps": peak, "peak_source": kind},
                        "k_pre": {"avg_ms": pre_ms, "source": "phase trace of the same steps (block 0 stamps)",
                                  "bytes_per_atom_no_rebuild": pre_bytes,
                                  "achieved_GBps": pre_bytes * n / (pre_ms * 1e-3) / 1e9 if pre_ms > 0 else None,
                                  "peak_GBps": peak},
                        "k_build_list": {"ms_per_rebuild": list_us / max(phases["rebuild_launches"], 1.0) * 1e-3,
                                         "ms_per_step": list_us / steps_t * 1e-3},
                        "k_pre_and_k_build_list_events_avg_ms": p_ms},
            "k_pre_phases_us_per_step": {k: v / steps_t for k, v in phases.items()
                                         if k not in ("launches", "rebuild_launches")}}
    print(json.dumps(line), flush=True)


def make_ensemble(nrep=512, seed=2024):
    """512 replicas: n^3 atoms on a simple-cubic lattice, n log-uniform in
    [4, 40]; rho* uniform in [0.01, 0.9]; T* uniform in [0.5, 2.0]; seeded
    velocities; each replica its own box, Berendsen T target T* and P target
    near its ideal-gas pressure rho* T*."""
    from moldyn_gb300.initializer import UnitCell, lattice_positions, maxwell_boltzmann
    rng = np.random.default_rng(seed)
    ns = np.rint(np.exp(rng.uniform(np.log(4), np.log(40), nrep))).astype(int)
    rho = rng.uniform(0.01, 0.9, nrep)
    tst = rng.uniform(0.5, 2.0, nrep)
    pos, vel, boxes, offs = [], [], [], [0]
    for r in range(nrep):
        a = rho[r] ** (-1.0 / 3.0)
        p = lattice_positions(UnitCell.U, (ns[r],) * 3, a)
        pos.append(p)
        vel.append(maxwell_boltzmann(len(p), tst[r] * 100.0 / K_B, 1.0, seed * 1000 + r))
        boxes.append(np.full(3, ns[r] * a))
        offs.append(offs[-1] + len(p))
    p0 = rho * tst * rng.uniform(0.8, 1.2, nrep)
    return (np.array(offs), np.concatenate(pos), np.concatenate(vel), np.array(boxes), ns, rho, tst, p0)


def run_ensemble(args):
    import torch
    from moldyn_gb300.engine import Engine
    from moldyn_gb300.initializer import Barostat, Thermostat
    from moldyn_gb300.sharding import max_over_ranks, replica_cost, shard
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    offs, pos, vel, boxes, ns, rho, tst, p0 = make_ensemble()
    n_all = len(pos)
    # replicas are independent: each rank integrates its own cost-balanced share
    mine = shard(replica_cost(ns ** 3, rho, 2.5 + SKIN), world)[rank]
    sel = np.concatenate([np.arange(offs[r], offs[r + 1]) for r in mine])
    pos, vel = pos[sel], vel[sel]
    offs = np.cumsum([0] + [int(offs[r + 1] - offs[r]) for r in mine])
    boxes, ns, rho, tst, p0 = boxes[mine], ns[mine], rho[mine], tst[mine], p0[mine]
    n, nrep = len(pos), len(offs) - 1
    t0s = tst * 100.0 / K_B
    res = {}
    # the mixed path with the skin chosen per size class by the engine, then
    # the same with the fixed 0.3 sigma skin, and the plain FP64 path
    for leg, prec, skin in (("mixed", "mixed", -1.0), ("mixed_fixed_skin", "mixed", SKIN), ("fp64", "fp64", SKIN)):
        e = Engine(precision=prec, skin=skin, persistent=True, graph_steps=50, **LIST_KW)
        e.set_potential(0, 0, 1.0, 1.0)
        e.upload_ensemble(offs, np.zeros(n, dtype=np.uint16), pos, vel, [1.0], boxes)
        e.compute_forces()
        ths = [Thermostat.Berendsen(0.5) for _ in range(nrep)]
        bas = [Barostat.Berendsen(1.0, 5.0) for _ in range(nrep)]
        e.ensemble_set_coupling(ths, t0s, bas, p0)
        steps = args.steps if prec == "mixed" else max(50, min(args.steps, args.fp64_steps or 50))
        e.ensemble_step(50, DT)            # warm-up (and skin tuning), graph capture
        e.prepare_step(steps, DT)
        e.reset_stats()
        if dist is not None:
            dist.barrier()
        ms = max_over_ranks(_timed_steps(e, steps, DT, ensemble=True), dist, "cuda")
        st = e.stats()
        res[leg] = {"value": n_all * steps / (ms * 1e-3), "steps": steps, "ms_per_step": ms / steps,
                    "graph_launches": st.graph_launches, "rebuilds": st.rebuilds,
                    "threads_per_atom_by_size_class": {"<2048": st.class_threads_per_atom[0],
                                                       "2048-32767": st.class_threads_per_atom[1],
                                                       ">=32768": st.class_threads_per_atom[2]},
                    "skin_sigma_by_size_class": {"<2048": st.class_skin[0], "2048-32767": st.class_skin[1],
                                                 ">=32768": st.class_skin[2]},
                    "skin": "tuned per size class" if skin < 0 else f"fixed {skin}",
                    "replicas_by_size_class": list(st.class_replicas)}
        e.close()
    if rank != 0:
        return
    line = {"metric": METRIC, "value": res["mixed"]["value"], "unit": "atom-steps/s", "n_gpus": world,
            "steps": res["mixed"]["steps"], "higher_is_better": True, "dtype": "f32/i64-fixed/f64",
            "scaling": "strong", "data": "synthetic: 512 seeded replicas (simple-cubic lattices)",
            "config": {"workload": "ensemble_512_replicas", "replicas": 512, "atoms": int(n_all),
                       "replicas_on_rank0": nrep,
                       "atoms_min_max_mean": [int(ns.min() ** 3), int(ns.max() ** 3), float((ns ** 3).mean())],
                       "graph_steps": 50, "persistent_force_kernel": True,
                       "mixed": res["mixed"], "mixed_fixed_skin": res["mixed_fixed_skin"],
                       "fp64_plain_path": res["fp64"],
                       "mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"]}}
    print(json.dumps(line), flush=True)


def run_splat(args):
    """Headless render of the 1M-atom box at 1920x1080 (the GUI viewer's
    shading through mdgb_splat): frames/s end to end through the C ABI (host
    particle buffer in, host image out), and the CPU oracle on a small frame."""
    from moldyn_gb300 import render as rnd
    from oracle import splat_ref
    pos, vel, box = make_system(seed=7)
    n = len(pos)
    parts = np.zeros((n, 12), dtype=np.float32)
    parts[:, 0:3] = pos
    parts[:, 3] = 1.0
    parts[:, 4:7] = vel
    parts[:, 7] = 1.0
    parts[:, 8] = 1.0
    parts[:, 9] = 0.5
    parts[:, 10] = np.arange(n) % 3
    w, h = 1920, 1080
    cam = rnd.framing_camera(box, w, h)
    prm = rnd.splat_params(cam, rnd.MODE_SPEED, speed_range=(0.0, 2.5), box=box)
    for _ in range(args.warmup):
        rnd.splat(parts, prm, w, h)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        img = rnd.splat(parts, prm, w, h)
    dt = (time.perf_counter() - t0) / args.steps
    # oracle: a 64x36 frame of the first 2000 particles, scaled to the same work
    sub = parts[:2000]
    cam_s = rnd.framing_camera(box, 64, 36)
    t0 = time.perf_counter()
    splat_ref.render(sub, {"view_pos": cam_s.uniform()[0], "view": cam_s.uniform()[1], "proj": cam_s.uniform()[2],
                           "mode": 1, "box": box, "grange": (0.0, 2.5), "gradient": rnd.DEFAULT_GRADIENT}, 64, 36)
    t_cpu = time.perf_counter() - t0
    cpu_pairs_per_s = 64 * 36 * 2000 / t_cpu
    line = {"metric": "headless frames/s, 1M LJ atoms at 1920x1080 (GUI shading)", "value": 1.0 / dt,
            "unit": "frames/s", "higher_is_better": True, "steps": args.steps, "warmup": args.warmup,
            "dtype": "f32", "data": "synthetic: seeded FCC 1M-atom liquid, radius 0.5 sigma",
            "config": {"workload": "splat_1m_1080p", "atoms": n, "width": w, "height": h, "mode": "speed gradient",
                       "box_edges": True, "lit_pixels": int((img[:, :, :3].sum(axis=2) > 0.05).sum())},
            "e2e": {"value": 1.0 / dt, "unit": "frames/s", "h2d_bytes_per_step": int(parts.nbytes),
                    "d2h_bytes_per_step": int(w * h * 16)},
            "cpu_baseline": {"value": cpu_pairs_per_s, "unit": "pixel-particle tests/s", "cores": 1, "kind": "port",
                             "sample": "oracle/splat_ref.py, 64x36 frame x 2000 particles, every pixel against every particle"}}
    print(json.dumps(line), flush=True)


def run_drift(args):
    """256,000 atoms (FCC 40^3 cells), NVE at dt* 0.005: total-energy drift of
    the FP32-naive, mixed (FP32 + fixed point) and FP64 paths."""
    global CELLS
    CELLS = (40, 40, 40)
    from moldyn_gb300.engine import Engine
    pos, vel, box = make_system(seed=55)
    n = len(pos)
    out = {}
    for prec in ("fp32_naive", "mixed", "fp64"):
        # every variant runs the same steps unless --fp64-steps shortens the FP64 one
        steps = args.steps if prec != "fp64" or not args.fp64_steps else min(args.steps, args.fp64_steps)
        every = max(1, steps // 100)
        e = Engine(precision=prec, skin=SKIN)
        e.set_potential(0, 0, 1.0, 1.0)
        e.upload(np.zeros(n, dtype=np.uint16), pos, vel, [1.0], box)
        e.compute_forces()
        es, ts, ps = [], [], []
        t0 = time.perf_counter()
        for k in range(0, steps + 1, every):
            if k:
                e.step(every, DT)
            m = e.macro(0)
            es.append(m["kinetic_energy"] + m["potential_energy"])
            ts.append(m["temperature"] * K_B / 100.0)
            ps.append(m["pressure"])
        wall = time.perf_counter() - t0
        es = np.array(es)
        x = np.arange(len(es)) * every * DT
        slope = float(np.polyfit(x, es / n, 1)[0]) if len(es) > 2 else 0.0
        out[prec] = {"steps": steps, "E0_per_atom": float(es[0] / n),
                     "drift_per_atom_per_tau": slope,
                     "rel_change": float((es[-1] - es[0]) / abs(es[0])),
                     "max_rel_dev": float(np.abs(es - es[0]).max() / abs(es[0])),
                     "T_star_mean": float(np.mean(ts)), "P_star_mean": float(np.mean(ps)),
                     "wall_s": wall}
        e.close()
    line = {"metric": "NVE energy drift (per atom per tau*), 256k LJ atoms", "value": out["mixed"]["drift_per_atom_per_tau"],
            "unit": "eps/(atom tau)", "higher_is_better": False,
            "config": {"workload": "drift_256k_nve", "atoms": n, "dt_star": DT, "variants": out,
                       "mixed_over_fp64_drift": (abs(out["mixed"]["drift_per_atom_per_tau"]) /
                                                 max(abs(out["fp64"]["drift_per_atom_per_tau"]), 1e-30))}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=None,
                    help="steps of the plain FP64 leg (default: 50 for lj1m and ensemble; drift: all steps)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--cells", default=None,
                    help="FCC unit cells (default 50,50,100 for lj1m, 100,100,200 for lj8m; profiling uses smaller boxes)")
    ap.add_argument("--legs", default="all", choices=["all", "mixed"],
                    help="'mixed' runs only the timed mixed leg (for profiler captures)")
    ap.add_argument("--trace", action="store_true", help="with --legs mixed: per-phase times of the step kernel")
    ap.add_argument("--direct-list", action="store_true",
                    help="lj1m and ensemble: the direct Verlet-list build (every cell against 27 cells) instead of the paired one")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                    help="with --legs mixed: the path whose steps are timed (profiler captures)")
    ap.add_argument("--tpa", type=int, default=0, help="threads per atom of the lj1m mixed leg (0: autotune)")
    ap.add_argument("--graph-steps", type=int, default=64,
                    help="lj1m: time the mixed path with chunks of this many steps replayed as CUDA graphs "
                         "(<= 1: eager launches with per-launch events)")
    ap.add_argument("--workload", default="lj1m", choices=["lj1m", "argon", "lj8m", "ensemble", "drift", "splat"],
                    help="lj1m: the headline 1M-atom box (default); the others are the remaining configurations")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    global CELLS
    if args.direct_list:
        LIST_KW["direct_list"] = True
    if args.cells:
        CELLS = tuple(int(c) for c in args.cells.split(","))
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "lj1m":
        run_ours(args)
    else:
        {"argon": run_argon, "lj8m": run_lj8m, "ensemble": run_ensemble, "drift": run_drift,
         "splat": run_splat}[args.workload](args)


if __name__ == "__main__":
    main()
