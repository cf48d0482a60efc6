"""Benchmark: simulated seconds per wall second of the ensemble forward run.

Workload (per GPU): the 256-member uneven ensemble of the data-assimilation
forward step -- members drawn with seeds 1000+m (30..80-cell square fractal
DEMs, 10..20 layers, sampled van Genuchten soils, water table 0.5..2 m),
1 simulated day each, Picard at TOLUNS = 1e-6 m.  One bench "step" replays
the whole ensemble day from the initial condition.

  value     device-timed throughput (CUDA events on the solver stream) of the
            batched path: FP32 assembly + column-line-preconditioned FP32 PCG
            inside the FP64 residual/refinement loop, all members in one
            launch sequence (one CUDA graph per Picard iteration, the PCG
            loop as a device-driven conditional node), inputs resident in HBM.
  e2e       the same through the public Python API with host buffers: each
            step uploads every member's initial heads from pinned memory
            (set_state), runs, and reads every member's final heads back.
  plain_gpu the reference's method on the GPU (FP64, IC(0)-PCG), one member
            at a time, over a sample of members.
  learned_preconditioner  the learned column-line factor on the CPU
            sample's members and window (train pass, then solve pass with
            plain fallback) beside the same launch-by-launch path without it.
  schedule  the autotuner's choice (assembly resident blocks per SM, SpMV
            blocks per SM), timed on the warmed-up ensemble.
  roofline  the SpMV kernel (dominant Krylov kernel): algorithmic bytes of
            every launch in the timed region / the launches' durations, each
            taken on the device clock from its first block's start to its
            last block's end (CUDA events cannot be recorded inside the
            graph's conditional body), against the measured HBM copy
            bandwidth.
  cpu_baseline  the CPU oracle (serial C++ restatement of the reference
            Fortran) on a bounded sample: members 1000..1014 and 1036 for
            their first 30 simulated minutes, one process per host core;
            also with pyCATHY's default pool of cpu_count() - 5 workers.
  same_sample_gpu_vs_cpu  the GPU path on exactly that sample (same
            members, same window, device-timed) beside the CPU figure: the
            like-for-like ratio.  The day's throughput varies with simulated
            time (the first minutes run at the smallest time steps), so the
            whole-day value and the sample are different workloads.

--impl reference runs the CPU restatement of the reference's solver on the
host cores (the Fortran reference cannot be built: no Fortran compiler) on a
bounded sample of the same ensemble and prints the same metric.

Multi-GPU (torchrun): the ensemble holds 256 members per rank (seeds 1000..)
and is split into one shard per rank, greedy by mesh size
(pycathy_wrapper_gb300.shard); each rank runs its shard as one batched
solve, no collective on the data path; value = all members' simulated
seconds / max rank time (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "simulated s per wall s at 1e-6 m head tol: learned+batched vs plain GPU PCG"
UNIT = "sim-s/wall-s"


def _cases(nmem, rank, tmax, precond, world=1):
    """This rank's members: the ensemble holds nmem * world members (seeds
    1000..), split across the ranks greedy by mesh size (one shard per GPU,
    no collective on the data path)."""
    from pycathy_wrapper_gb300.inputs import config2_members
    cases = config2_members(nmem * world, tmax=tmax, base_seed=1000)
    if world > 1:
        from pycathy_wrapper_gb300.shard import member_nodes, shard_of
        cases = [cases[m] for m in shard_of(member_nodes(cases), rank, world)]
    for c in cases:
        c.parm.precond = precond
    return cases


# ---------------------------------------------------------------------------
# Bounded sample for the CPU baseline, the reference arm and the GPU run on
# the same sample: the first 15 members and member 36 (seed 1036, which fails
# later in the day: a hard member), each for its first SAMPLE_TMAX simulated
# seconds.
# ---------------------------------------------------------------------------
SAMPLE = list(range(15)) + [36]
SAMPLE_TMAX = 1800.0


def _sample_cases(nmem, tmax, precond):
    allc = _cases(nmem, 0, tmax, precond=precond)
    return [allc[i] for i in SAMPLE if i < len(allc)]


def _oracle_member(args):
    k, nmem, tmax = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    c = _sample_cases(nmem, tmax, precond=0)[k]
    o = O.Oracle(c)
    t0 = time.perf_counter()
    o.run()
    el = time.perf_counter() - t0
    sr = o.step_records()
    return (sr[-1]["time"] if sr else 0.0), el


def cpu_sample(nmem, tmax, cores):
    """The CPU restatement of the reference solver on the sample, one member
    per worker process (pyCATHY's DA runs one ./cathy per member in a
    process pool); returns simulated s per wall s, wall s, simulated s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    n = len(_sample_cases(nmem, tmax, precond=0))
    jobs = [(k, nmem, tmax) for k in range(n)]
    t0 = time.perf_counter()
    with ctx.Pool(processes=max(1, cores)) as pool:
        res = pool.map(_oracle_member, jobs)
    wall = time.perf_counter() - t0
    sim = sum(r[0] for r in res)
    return sim / wall, wall, sim


def gpu_sample(nmem, tmax, device, graphs):
    """The GPU path on the same sample (device-timed, one batched solve)."""
    from pycathy_wrapper_gb300.api import Simulation
    cases = _sample_cases(nmem, tmax, precond=2)
    with Simulation(cases, precision=1, device=device, graphs=graphs) as s:
        s.run(20)  # warm-up: the first steps of every member
        s.reset()
        a = s.stats()["gpu_ms"]
        s.run()
        dev = (s.stats()["gpu_ms"] - a) / 1000.0
        sim = sum(s.state(m)[1] for m in range(s.nmembers))
    return sim / dev, dev, sim


def learned_sample(nmem, tmax, device):
    """The learned column-line preconditioner on the bounded sample, against
    the same launch-by-launch path without it: one pass in training mode
    (mode 1: the network learns from the plain solver's Krylov pairs; heads
    are the plain ones), then a pass that solves with the trained factor
    (mode 2, plain factor as fallback).  Device-timed; returns both
    throughputs and the mean PCG iterations per solve."""
    from pycathy_wrapper_gb300.api import Simulation
    from pycathy_wrapper_gb300.learned import LearnedPreconditioner, init_params
    cases = _sample_cases(nmem, tmax, precond=2)

    def one(lp, mode):
        with Simulation(cases, precision=1, device=device, graphs=False) as s:
            if lp is not None:
                s.attach_learned(lp, mode=mode)
            a = s.stats()
            s.run()
            b = s.stats()
            dev = (b["gpu_ms"] - a["gpu_ms"]) / 1000.0
            sim = sum(s.state(m)[1] for m in range(s.nmembers))
            lin = b["lin_iters"] - a["lin_iters"]
            nl = b["nl_iters"] - a["nl_iters"]
            st = s.learned_stats() if lp is not None else None
        return dict(value=sim / dev, device_s=dev, lin_per_nl=lin / max(nl, 1)), st

    plain, _ = one(None, 0)
    with LearnedPreconditioner(init_params(0), device=device, lr=1e-3) as lp:
        train, tst = one(lp, 1)
        use, ust = one(lp, 2)
    return {"unit": UNIT, "sample": "the CPU sample's members and window, launch by launch",
            "plain": plain, "training_pass": dict(train, train_steps=tst["train_steps"],
                                                  last_loss=tst["last_loss"]),
            "learned": dict(use, learned_solves=ust["learned_solves"],
                            plain_solves=ust["plain_solves"],
                            learned_iters_per_solve=ust["learned_iters"] / max(ust["learned_solves"], 1),
                            plain_iters_per_solve=ust["plain_iters"] / max(ust["plain_solves"], 1)),
            "learned_over_plain": use["value"] / plain["value"]}


# ---------------------------------------------------------------------------
SPMV_DRAM_PER_ALG_BYTE = 356.1 / 362.4


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler during the timed region."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", os.environ.get("LOCAL_RANK", "0"),
                 f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([t.strip() for t in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
                for k, v in zip(names, r[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(k)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, ws):
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def allsum(x, ws):
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())
    return x


# ---------------------------------------------------------------------------
def run_reference(args):
    rank, ws = dist_init()
    if rank != 0:
        barrier(ws)
        return
    cores = os.cpu_count() or 1
    vals, walls = [], []
    # warm-up steps (process start-up, page cache) run a short sample; the
    # timed steps run the bounded sample itself
    for i in range(args.warmup + args.steps):
        tmax = args.cpu_tmax if i >= args.warmup else min(args.cpu_tmax, 120.0)
        v, wall, sim = cpu_sample(args.members, tmax, cores)
        if i >= args.warmup:
            vals.append(v)
            walls.append(wall)
    value = sum(vals) / len(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sum(walls) / len(walls), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"ensemble{args.members}_day", "members": args.members,
                   "tmax_s": args.tmax, "sample_members": [1000 + i for i in SAMPLE]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"members {[1000 + i for i in SAMPLE]}, first "
                                   f"{args.cpu_tmax:g} simulated s each, one process per core "
                                   f"(CPU restatement of the reference Fortran, -O2; gfortran "
                                   f"absent)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(ws)


def run_large(args):
    """The other configurations at their stated sizes, on the FP32 path:
    config 1 (one 200x200-cell fractal DEM, 30 layers, lognormal Ks, rain
    pulse, 2 simulated days, column-line PCG) and config 4 (32 members of
    300x300 cells and 25 layers, ponded infiltration, Newton with FP32
    BiCGSTAB inside the FP64 loop; its first `--steps` time steps, the
    build and the device memory are the figures of interest)."""
    from pycathy_wrapper_gb300.api import Simulation
    from pycathy_wrapper_gb300.inputs import config1, config4_member, with_vegetation
    import torch
    if args.workload == "config1":
        cases = [config1(tmax=172800.0)]
        cases[0].parm.precond = 2
        steps = 0
    elif args.workload == "vegetated":
        # the bench's ensemble with the Feddes root-water uptake switched on
        # (SCF = 1, two vegetation types, rain then evaporation): the cost of
        # ETRAN at ensemble scale, on the bench's FP32 graph path
        cases = [with_vegetation(c) for c in _cases(args.members, 0, args.tmax, precond=2)]
        steps = 0
    else:
        nm = min(args.members, 32)  # 32 members by default; fewer for a profiling run
        cases = [config4_member(300, 25, seed=k, tmax=43200.0) for k in range(nm)]
        steps = max(args.steps, 1)
    free0 = torch.cuda.mem_get_info()[0]
    t0 = time.perf_counter()
    with Simulation(cases, precision=1,
                    graphs=args.workload != "config4" and not args.no_graphs) as s:
        build_s = time.perf_counter() - t0
        dev_gb = (free0 - torch.cuda.mem_get_info()[0]) / 1e9
        a = s.stats()
        s.run(steps)
        b = s.stats()
        dev = (b["gpu_ms"] - a["gpu_ms"]) / 1e3
        sim = sum(s.state(m)[1] for m in range(s.nmembers))
        st = [s.state(m)[3] for m in range(s.nmembers)]
        nodes = int(sum(z["n"] for z in s.sizes))
        nnz = int(sum(z["nnz"] for z in s.sizes))
        line = {"metric": METRIC, "value": sim / dev, "unit": UNIT, "n_gpus": 1,
                "workload": args.workload, "members": len(cases), "nodes_total": nodes,
                "nnz_total": nnz, "device_s": dev, "simulated_s": sim,
                "nl_iterations": b["nl_iters"] - a["nl_iters"],
                "lin_iterations": b["lin_iters"] - a["lin_iters"],
                "finished": int(sum(1 for v in st if v == 1)), "build_s": build_s,
                "device_gb": dev_gb, "steps": steps if steps else "to TMAX",
                "dtype": "f32+f64", "data": "synthetic (seeded)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--warmup-member-steps", type=int, default=50,
                    help="accepted time steps per member in each warm-up pass")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--tmax", type=float, default=86400.0)
    ap.add_argument("--cpu-tmax", type=float, default=SAMPLE_TMAX,
                    help="simulated seconds per member in the bounded CPU sample")
    ap.add_argument("--plain-members", type=int, default=4)
    ap.add_argument("--no-graphs", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--only", default="",
                    help="comma-separated member indices: run only these (profiling)")
    ap.add_argument("--workload", default="ensemble",
                    choices=["ensemble", "config1", "config4", "vegetated"],
                    help="config1 / config4: the single large mesh (200x200x30, 2 simulated days) "
                         "or the 32-member Newton batch (300x300x25 each, first steps) at their "
                         "stated sizes; vegetated: the ensemble day with the Feddes sink; a "
                         "line of its own, not the bench line")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "ensemble":
        return run_large(args)
    rank, ws = dist_init()
    # CPU baseline first (spawned pool, before any GPU context)
    cpu = cpu_pyc = None
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count() or 1
        v, wall, sim = cpu_sample(args.members, args.cpu_tmax, cores)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"members {[1000 + i for i in SAMPLE]} x first {args.cpu_tmax:g} "
                         f"simulated s, one process per core, {wall:.1f} s wall"}
        # pyCATHY's default DA pool size (cathy_DA.py: cpu_count() - 5)
        wk = max(1, cores - 5)
        v2, wall2, _ = cpu_sample(args.members, args.cpu_tmax, wk)
        cpu_pyc = {"value": v2, "unit": UNIT, "cores": wk,
                   "sample": f"same sample, {wk} worker processes, {wall2:.1f} s wall"}
    import numpy as np
    from pycathy_wrapper_gb300.api import Simulation
    dev_id = int(os.environ.get("LOCAL_RANK", "0"))
    # the GPU path on the CPU baseline's sample (same members, same window)
    like = None
    if rank == 0 and cpu is not None:
        vg, devs, _ = gpu_sample(args.members, args.cpu_tmax, dev_id, not args.no_graphs)
        like = {"sample": cpu["sample"].split(", one process")[0], "gpu": vg, "cpu": cpu["value"],
                "cpu_cores": cpu["cores"], "gpu_over_cpu": vg / cpu["value"], "unit": UNIT,
                "gpu_s": devs}
    cases = _cases(args.members, rank, args.tmax, precond=2, world=ws)
    if args.only:
        # a profiling run on chosen members of the ensemble (e.g. one tail
        # member), not a bench line
        cases = [cases[int(k)] for k in args.only.split(",")]
    sim = Simulation(cases, precision=1, device=dev_id, graphs=not args.no_graphs)
    nodes_total = int(sum(s["n"] for s in sim.sizes))
    nnz_total = int(sum(s["nnz"] for s in sim.sizes))
    # q = A p with the dots p.q, p.r: values and columns, then per row its
    # pointer, p, q and r
    spmv_full_bytes = 8.0 * nnz_total + 16.0 * nodes_total
    # warm-up: partial passes of the same workload (every member's first
    # time steps: every kernel runs, the graphs of the early member sets are
    # built); untimed
    for _ in range(args.warmup):
        sim.reset()
        sim.run(args.warmup_member_steps)
    # the assembly (the dominant kernel of the full-batch iterations) on the
    # whole ensemble: mean of 20 launches between CUDA events, inputs far
    # larger than L2 (no flush needed)
    # the schedule: resident blocks per SM of the assembly, stream-SpMV grid
    # (project autotuner, cached per GPU), then the assembly's own timing:
    # both on every member after its first 5 accepted steps (all members
    # still running)
    sim.reset()
    sim.run(5)
    sched = sim.autotune(10)
    asm_ms, asm_bytes, asm_rows = sim.time_assembly(20)

    def reached():
        # simulated seconds actually covered (members that fail stop early)
        return sum(sim.state(m)[1] for m in range(sim.nmembers))
    # ---- device-timed steps ----
    clocks = Clocks()
    barrier(ws)
    st0 = sim.stats()
    sim.profile(1)
    clocks.start()
    t0 = time.perf_counter()
    sim_seconds = 0.0
    for _ in range(args.steps):
        sim.reset()
        sim.run()
        sim_seconds += reached()
    wall = time.perf_counter() - t0
    ck = clocks.stop()
    spmv_ms, spmv_n, spmv_bytes = sim.profile(0)
    st1 = sim.stats()
    dev_s = (st1["gpu_ms"] - st0["gpu_ms"]) / 1000.0
    dev_s = allmax(dev_s, ws)
    barrier(ws)
    total_sim = allsum(sim_seconds, ws)
    value = total_sim / dev_s
    launches = st1["launches"] - st0["launches"]
    nl = st1["nl_iters"] - st0["nl_iters"]
    lin = st1["lin_iters"] - st0["lin_iters"]
    # check: every member finished its day
    fin = [sim.state(m)[3] for m in range(sim.nmembers)]
    # ---- e2e through the public API with pinned host buffers ----
    try:
        import torch
        pin = lambda n: torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    except Exception:
        pin = lambda n: np.empty(n)
    ic = []
    sim.reset()
    for m in range(sim.nmembers):
        p, _, _, _ = sim.state(m)
        buf = pin(len(p))
        buf[:] = p
        ic.append(buf)
    out = [pin(sim.sizes[m]["n"]) for m in range(sim.nmembers)]
    h2d = sum(b.nbytes for b in ic)
    d2h = sum(b.nbytes for b in out)
    barrier(ws)
    t0 = time.perf_counter()
    e2e_sim = 0.0
    for _ in range(args.e2e_steps):
        sim.reset()
        for m in range(sim.nmembers):
            sim.set_state(m, ic[m], cases[m].parm.deltat, cases[m].parm.deltat)
        sim.run()
        for m in range(sim.nmembers):
            out[m][:], tm, _, _ = sim.state(m)
            e2e_sim += tm
    e2e_wall = allmax(time.perf_counter() - t0, ws)
    e2e = {"value": allsum(e2e_sim, ws) / e2e_wall, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": args.e2e_steps}
    sim.close()
    # ---- plain GPU path (FP64 IC(0)-PCG, unbatched) on a sample ----
    plain = None
    if rank == 0 and not args.no_plain:
        allc = _cases(args.members, 0, args.tmax, precond=0)
        stride = max(1, args.members // max(args.plain_members, 1))
        pick = list(range(0, args.members, stride))[: args.plain_members]
        tot_t, tot_s = 0.0, 0.0
        for k in pick:
            with Simulation(allc[k], precision=0) as s1:
                a = s1.stats()["gpu_ms"]
                s1.run()
                tot_t += (s1.stats()["gpu_ms"] - a) / 1000.0
                tot_s += s1.state(0)[1]
        plain = {"value": tot_s / tot_t, "unit": UNIT,
                 "sample": f"members {pick} one at a time, FP64 IC(0)-PCG, 1 simulated day"}
    learned = None
    if rank == 0 and not args.no_learned:
        learned = learned_sample(args.members, args.cpu_tmax, dev_id)
    if rank != 0:
        return
    peak, peak_kind = _peaks()
    achieved = (spmv_bytes / 1e9) / (spmv_ms / 1e3) if spmv_ms > 0 else None
    # DRAM bytes per algorithmic byte of one full-batch k_spmv_stream launch
    # (direction update + product) from an ncu capture of the 48-member
    # ensemble: 356.1 MB read + written for 362.4 MB algorithmic; scaled to
    # the average launch of this run by its algorithmic bytes
    traffic = SPMV_DRAM_PER_ALG_BYTE * spmv_bytes / spmv_n if spmv_n else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded ensemble: fractal DEMs, sampled van Genuchten soils)",
        "config": {"workload": (f"ensemble{args.members}_day" if not args.only else
                                f"ensemble{args.members}_members_{args.only}_day"),
                   "members": args.members,
                   "tmax_s": args.tmax, "nodes_total": nodes_total, "nnz_total": nnz_total,
                   "warmup": f"{args.warmup} partial passes ({args.warmup_member_steps} accepted "
                             f"steps per member)",
                   "precision": "fp32 matrix/Krylov, fp64 residual+refinement",
                   "cuda_graphs": not args.no_graphs,
                   "preconditioner": "column-line (vertical tridiagonal) block Jacobi",
                   "l2": "inputs larger than L2 (ensemble matrix > 1.5 GB)",
                   "parallelism": f"members sharded per rank x{ws}",
                   "schedule": sched},
        "e2e": e2e,
        "gpu_launches": launches,
        "nl_iterations": nl, "lin_iterations": lin,
        "members_finished": int(sum(1 for f in fin if f == 1)),
        "members_failed": [i for i, f in enumerate(fin) if f == 2],
        "wall_s_timed": wall,
        "roofline": {"bound": "hbm", "kernel": "k_spmv_stream",
                     "timing": "per launch on the device clock (first block start to last "
                               "block end), every SpMV of the timed region",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "peak_source": peak_kind, "traffic": traffic,
                     "launches": spmv_n, "alg_bytes_per_launch": spmv_bytes / max(spmv_n, 1)},
        "roofline_assembly": {
            "bound": "hbm", "kernel": "k_assemble_picard_f32",
            "timing": f"mean of 20 launches over all {args.members} members after their first "
                      f"5 steps, CUDA events",
            "achieved": asm_bytes / 1e9 / (asm_ms / 1e3), "peak": peak, "unit": "GB/s",
            "frac": asm_bytes / 1e9 / (asm_ms / 1e3) / peak, "peak_source": peak_kind,
            "alg_bytes_per_launch": asm_bytes, "rows": asm_rows, "ms_per_launch": asm_ms},
        "roofline_spmv_full_batch": {
            "bound": "hbm", "kernel": "k_spmv_stream<kSpmvPlain>",
            "timing": f"the autotuner's best mean over 10 launches on all {args.members} members "
                      f"after their first 5 steps, CUDA events",
            "achieved": spmv_full_bytes / 1e9 / (sched["spmv_ms"] / 1e3), "peak": peak,
            "unit": "GB/s", "frac": spmv_full_bytes / 1e9 / (sched["spmv_ms"] / 1e3) / peak,
            "peak_source": peak_kind, "alg_bytes_per_launch": spmv_full_bytes,
            "ms_per_launch": sched["spmv_ms"]},
        "cpu_baseline": cpu,
        "cpu_baseline_pycathy_workers": cpu_pyc,
        "same_sample_gpu_vs_cpu": like,
        "plain_gpu": plain,
        "speedup_vs_plain_gpu": (value / plain["value"]) if plain else None,
        "learned_preconditioner": learned,
        "clocks": ck,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
