#!/usr/bin/env python
"""Throughput benchmark of the single-level incompressible advance.

Workload: neutral ABL LES, 256 x 256 x 128 cells on 5120 x 5120 x 1280 m (20 x 20 x 10 m cells),
FP64, Godunov PPM advection, MAC and nodal projections by geometric
multigrid, Smagorinsky Cs = 0.135, geostrophic (8 m/s) + Coriolis forcing,
wall-model bottom, slip top, CFL 0.9, log-law start with seeded +-0.5 m/s
noise below 300 m (synthetic input: no dataset exists for this path).

One "step" is one iteration of the Evolve loop (compute_dt, pre-advance
work, ApplyPredictor with both projections).  The state (~6 GB) is larger
than L2 (129 MB), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank advances its own replica (the path is replicas-only
on one GPU each); value = all ranks' cell-steps / max rank time.  The
reference arm times the CPU restatement (the reference's own build cannot be
compiled: its AMReX / AMReX-Hydro submodules are absent) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s at 256^3 (FP64 vs mixed-precision at stated error) + adjoint/forward cost ratio"
UNIT = "Mcell-steps/s"
# the ABL box: 256 x 256 x 128 cells on 5120 x 5120 x 1280 m, i.e. 20 x 20 x 10 m cells
# (other --size values keep the cell size; --dz changes the vertical one)
ABL_DZ = 10.0
CPU_SAMPLE = (128, 128, 64)  # same dx, physics and deck as the workload, 1/8 of the cells
DATA = "synthetic (log-law + seeded uniform noise, SplitMix64 seed 42)"


def workload(dz):
    return ("ABL LES 256x256x128 FP64 (5120x5120x%g m: 20x20x%g m cells, Smagorinsky, geostrophic+Coriolis, wall model, CFL 0.9)"
            % (128 * dz, dz))


def workload_config(size, dz, world=1):
    """The `config` object both arms print (the workload, not a measurement)."""
    return {"workload": workload(dz), "cells": list(size), "cell_size_m": [20.0, 20.0, dz],
            "parallelism": "replicas" if world > 1 else "single GPU", "l2": "state larger than L2 (no flush)"}
# FP64 flops per algorithmic byte (an FMA counts 2) of the kernels that can dominate the FP64 step:
# nodal column sweep 20 flops per node (5 plane sums, 3 pair sums, 5 FMAs from the right-hand side,
# 1 FMA update) over 24 bytes; residual form 18; red-black update 10 flops over 16 bytes
FP64_FLOPS_PER_BYTE = {"(k_nd_col<T,0>)": 20.0 / 24.0, "(k_nd_col<double,1>)": 20.0 / 24.0, "(k_nd_col<T,2>)": 18.0 / 24.0,
                       "k_cc_gsrb<T>": 10.0 / 16.0}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision form of the same workload")
    p.add_argument("--c2-steps", type=int, default=100, help="steps of the FP64 / mixed-precision comparison")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint cost / gradient check (128x128x64, 3 disks)")
    p.add_argument("--no-mol", action="store_true", help="skip the MOL and Crank-Nicolson forms of the ABL workload")
    p.add_argument("--no-semi", action="store_true", help="skip the workload with MAC semicoarsening (mac_proj.do_semicoarsening)")
    p.add_argument("--c4", action="store_true",
                   help="only the production forward + adjoint run: 512x512x256 ABL, 16 disks, mixed forward, FP64 adjoint")
    p.add_argument("--c4-steps", type=int, default=200)
    p.add_argument("--c4-slots", type=int, default=12)
    p.add_argument("--c4-fd-h", default="1e-6,1e-8", help="finite-difference steps for the 2-disk gradient check")
    p.add_argument("--profile-all", action="store_true", help="print the per-kernel breakdown to stderr")
    p.add_argument("--size", default="256,256,128")
    p.add_argument("--dz", type=float, default=ABL_DZ, help="vertical cell size of the ABL workloads in m (20 m horizontal)")
    p.add_argument("--ref-budget", type=float, default=150.0,
                   help="reference arm: seconds of timed CPU steps after which it stops (at least one step; 0: no limit)")
    p.add_argument("--cpu-worker", default="", help=argparse.SUPPRESS)
    return p.parse_args()


# ---------------------------------------------------------------- replicas
def max_over_ranks(value, world, device="cuda"):
    """The slowest rank's time: every rank advances its own replica (the path
    does not shard), so the job ends when the last replica does."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as tdist
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells, steps, world, seconds):
    """Whole-job Mcell-steps/s: all replicas' cell-steps over the slowest rank's time."""
    return cells * steps * world / seconds / 1e6


# ---------------------------------------------------------------- CPU side
def cpu_worker(spec):
    """Runs in a child process: times the oracle.  spec = "warm,steps,repeats,nx,ny,nz,dz,budget[,case]":
    `repeats` fresh runs of the ABL deck on nx x ny x nz cells of 20 x 20 x dz m (or the 64^3
    Taylor-Green case, or the MOL form of the ABL deck), each timing `steps`
    Evolve steps after `warm` untimed ones, initialisation skipped.  A budget
    above 0 (seconds) ends a run's warm-up after a quarter of it and its timed
    steps once they have used it, after at least one."""
    parts = spec.split(",")
    warm, steps, repeats = int(parts[0]), int(parts[1]), int(parts[2])
    nx, ny, nz = int(parts[3]), int(parts[4]), int(parts[5])
    dz, budget = float(parts[6]), float(parts[7])
    case = parts[8] if len(parts) > 8 else ""
    from kynema_sgf_gb300 import decks
    from oracle.oracle import Oracle
    skip_init = "\nincflo.do_initial_proj = 0\nincflo.initial_iterations = 0\n"
    deck = decks.abl(nx, ny, nz, steps=10 ** 6, dz=dz) + skip_init
    if case == "tgv":
        nx = ny = nz = 64
        deck = decks.tgv(64, steps=10 ** 6)
    if case == "mol":
        deck = decks.mol(decks.abl(nx, ny, nz, steps=10 ** 6, cfl=0.45, dz=dz)) + skip_init
    runs = []
    for _ in range(repeats):
        o = Oracle(deck)
        t0 = time.perf_counter()
        for _ in range(warm):
            o.step()
            if budget > 0 and time.perf_counter() - t0 > 0.25 * budget:
                break
        per = []
        for _ in range(steps):
            t0 = time.perf_counter()
            o.step()
            per.append(time.perf_counter() - t0)
            if budget > 0 and sum(per) > budget:
                break
        runs.append(per)
        del o
    print(json.dumps({"runs": runs, "cells": nx * ny * nz}))


def cpu_model():
    """Host CPU model name and logical core count (lscpu, else /proc/cpuinfo)."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                name = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    name = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    import platform
    return {"model": name, "logical_cores": os.cpu_count(), "machine": platform.machine()}


def run_cpu(warm, steps, repeats=1, size=CPU_SAMPLE, case="", dz=ABL_DZ, budget=0.0):
    """Time the oracle on all host cores in a child process; returns (cells,
    per-run Mcell-steps/s list, per-run step times, cores)."""
    from oracle import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), OMP_PROC_BIND="spread", OMP_PLACES="cores")
    spec = "%d,%d,%d,%d,%d,%d,%r,%r" % ((warm, steps, repeats) + tuple(size) + (float(dz), float(budget))) + ("," + case if case else "")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-worker", spec],
                       capture_output=True, text=True, env=env, cwd=ROOT)
    if r.returncode != 0:
        raise RuntimeError("CPU baseline failed: " + r.stderr[-2000:])
    out = json.loads(r.stdout.strip().splitlines()[-1])
    cells = out["cells"]
    rates = [cells * len(per) / sum(per) / 1e6 for per in out["runs"]]
    return cells, rates, out["runs"], cores


def cpu_baseline_entry(warm, steps, repeats, size=CPU_SAMPLE, case="", what=None, dz=ABL_DZ):
    """The median over `repeats` fresh runs of the oracle's rate."""
    cells, rates, runs, cores = run_cpu(warm, steps, repeats, size, case, dz)
    nx, ny, nz = size if case != "tgv" else (64, 64, 64)
    what = what or ("CPU restatement (oracle/ks_oracle.cpp, g++ -O3 -fopenmp) on %dx%dx%d cells of the same ABL deck (same cell size "
                    "20x20x%g m and physics%s)" % (nx, ny, nz, dz, ", 1/8 of the cells" if (nx, ny, nz) == CPU_SAMPLE else ""))
    return {"value": statistics.median(rates), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%s; median of %d fresh runs, each %d timed Evolve steps after %d untimed, initialisation skipped"
                      % (what, repeats, steps, warm),
            "runs": [round(x, 4) for x in rates], "cpu": cpu_model()}


# ---------------------------------------------------------------- clocks
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- GPU side
def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel, algorithmic_bytes_per_launch):
    """DRAM bytes per launch of `kernel`, from the committed ncu summary: the
    captured launch's DRAM/algorithmic ratio scaled to this run's launches."""
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        ratio = t.get(kernel, {}).get("dram_to_algorithmic_ratio")
        return ratio * algorithmic_bytes_per_launch if (ratio and algorithmic_bytes_per_launch) else None
    except Exception:
        return None


def our_arm(args, rank, world, local_rank):
    import torch
    import kynema_sgf_gb300 as ks
    from kynema_sgf_gb300 import decks
    dist = world > 1
    if dist:
        import torch.distributed as tdist
    torch.cuda.set_device(local_rank)
    nx, ny, nz = (int(x) for x in args.size.split(","))
    sim = ks.Incflo(decks.abl(nx, ny, nz, steps=10 ** 9, dz=args.dz))
    sim.InitData()
    cells = sim.scalar("ncells")
    # warm-up; the last warm-up step times every kernel to pick the dominant one
    for w in range(args.warmup):
        if w == args.warmup - 1:
            sim.profile_kernels("*")
        sim.step()
    breakdown = sim.profile_report()
    # "(mg_coarse_graph)" times whole graph replays (many kernels), not one kernel
    dominant = max((k for k in breakdown if not k.startswith("(mg_")), key=lambda k: breakdown[k][1])
    if args.profile_all and rank == 0:
        tot = sum(v[1] for v in breakdown.values())
        for k, v in sorted(breakdown.items(), key=lambda kv: -kv[1][1]):
            sys.stderr.write("%-22s %6d launches %9.3f ms %5.1f%% %8.1f GB/s\n" % (k, v[0], v[1], 100 * v[1] / tot,
                                                                                  v[2] / (v[1] * 1e-3) / 1e9 if v[1] else 0))
    sim.profile_kernels(dominant)
    stream = torch.cuda.ExternalStream(sim.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local_rank)
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    l0 = sim.kernel_launches()
    mac_it, nod_it = [], []
    clocks.start()
    ev0.record(stream)
    for _ in range(args.steps):
        sim.step()
        mac_it.append(sim.scalar("mac_iters"))
        nod_it.append(sim.scalar("nodal_iters"))
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        tdist.barrier()
    launches = sim.kernel_launches() - l0
    div = divergence(sim)
    ms_max = max_over_ranks(ev0.elapsed_time(ev1), world)
    dom = sim.profile_report().get(dominant, (0, 0.0, 0.0))
    fp64_peak = ks.fma_peak(True)
    sim.profile_kernels("")
    value = replica_throughput(cells, args.steps, world, ms_max * 1e-3)

    # end to end through the public API: host inputs in, host result out
    e2e = None
    if not args.no_e2e:
        shapes = {f: sim.layout(f) for f in ("velocity", "gp", "p")}
        host = {f: torch.empty(int(torch.tensor(s).prod()), dtype=torch.float64, pin_memory=True) for f, s in shapes.items()}
        for f in host:
            sim.get_field(f, out=host[f])
        if dist:
            tdist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for f in ("velocity", "gp", "p"):
                sim.set_field(f, host[f])
            sim.step()
            sim.get_field("velocity", out=host["velocity"])
        torch.cuda.synchronize()
        el = max_over_ranks(time.perf_counter() - t0, world)
        hin = sum(host[f].numel() * 8 for f in host)
        e2e = {"value": replica_throughput(cells, args.steps, world, el), "unit": UNIT, "h2d_bytes_per_step": hin,
               "d2h_bytes_per_step": host["velocity"].numel() * 8}
    # the other forms of the workload: a failure of one is reported in its entry, and the
    # headline numbers above stand
    mixed = None
    if not args.no_mixed:
        del sim
        mixed = leg(c2_bench, args, torch, ks, decks, nx, ny, nz, world, rank, ms_max / args.steps)
    mol = None if args.no_mol else leg(mol_bench, args, torch, ks, decks, nx, ny, nz, world, rank)
    cn = None if args.no_mol else leg(cn_bench, args, torch, ks, decks, nx, ny, nz, world, rank)
    strat = None if args.no_mol else leg(stratified_bench, args, torch, ks, decks, nx, ny, nz, world, rank)
    adj = None if args.no_adjoint else leg(adjoint_bench, args, torch, ks, decks)
    tgv = leg(tgv_bench, args, torch, ks, decks)
    # last, so that no number above depends on it
    semi = None if (args.no_semi or world > 1) else semi_bench(args, torch, ks, decks, nx, ny, nz, world, rank)
    return dict(value=value, ms=ms_max, cells=cells, launches=launches, dominant=dominant, dom=dom, clocks=clk, e2e=e2e, fp64_peak=fp64_peak, div=div,
                mac=statistics.mean(mac_it), nodal=statistics.mean(nod_it), size=(nx, ny, nz), mixed=mixed, adjoint=adj, tgv=tgv, mol=mol, cn=cn, strat=strat,
                semi=semi)


def tgv_bench(args, torch, ks, decks):
    """The reference's own CPU-runnable case: Taylor-Green vortex 64^3, Re 1600,
    CFL 0.5, 20 timed steps after --warmup."""
    tg = ks.Incflo(decks.tgv(64, steps=10 ** 6))
    tg.InitData()
    for _ in range(args.warmup):
        tg.step()
    tstream = torch.cuda.ExternalStream(tg.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(tstream)
    for _ in range(20):
        tg.step()
    ev1.record(tstream)
    torch.cuda.synchronize()
    tms = ev0.elapsed_time(ev1) / 20
    del tg
    return {"workload": "Taylor-Green vortex 64^3, Re 1600, CFL 0.5, FP64, 20 timed steps", "value": 64 ** 3 / (tms * 1e-3) / 1e6,
            "unit": UNIT, "ms_per_step": tms}


def leg(fn, *a):
    """Run one secondary leg of the bench; an exception becomes its entry."""
    try:
        return fn(*a)
    except Exception as e:  # reported in the line, never silently replaced
        return {"failed": "%s: %s" % (type(e).__name__, str(e)[:300])}


def divergence(sim):
    """Post-projection divergence of the current state.  The MAC projection is
    exact: max|div u_mac| is its FP64 residual.  The nodal projection is an
    approximate projection: the nodal divergence of the cell velocity is
    truncation-sized, and the solve's own divergence is its final residual.
    Relative forms scale by max|u| / min(dx, dy, dz)."""
    return {"mac_divu_rel": sim.scalar("mac_divu_rel"), "mac_divu": sim.scalar("mac_divu"),
            "nodal_residual_rel": sim.scalar("nodal_res") / max(sim.scalar("nodal_res0"), 1e-300),
            "mac_residual_rel": sim.scalar("mac_res") / max(sim.scalar("mac_res0"), 1e-300),
            "cell_nodal_divu_rel": sim.scalar("divu_rel"), "cell_nodal_divu": sim.scalar("divu")}


def kernel_table(rep, top=12):
    tot = sum(v[1] for v in rep.values())
    rows = sorted(rep.items(), key=lambda kv: -kv[1][1])[:top]
    return [[k, v[0], round(v[1], 3), round(v[1] / tot, 4), round(v[2] / (v[1] * 1e-3) / 1e9, 1) if v[1] else None] for k, v in rows]


def c2_bench(args, torch, ks, decks, nx, ny, nz, world, rank, fp64_ms_main):
    """The mixed-precision form of the ABL workload against its FP64 form: both
    advance the same deck from the same initial state for --c2-steps steps.
    The FP64 fields after those steps are the reference for the mixed form's
    errors (velocity, pressure, pressure gradient; relative L2 and max-norm);
    both forms' post-projection divergence is taken after every step.  Time:
    CUDA events around each step (the divergence reads between steps are not
    timed); throughput over the last --steps steps (dt at the CFL limit) and
    over all steps.  The mixed form's dominant kernel is timed over the last
    --steps steps for its roofline."""
    nsteps = max(args.c2_steps, args.steps + 1)
    peak, peak_kind = peaks()
    res = {}
    for form in ("fp64", "mixed"):
        deck = decks.abl(nx, ny, nz, steps=10 ** 9, dz=args.dz) + ("\nks.precision = mixed\n" if form == "mixed" else "")
        sim = ks.Incflo(deck)
        sim.InitData()
        cells = sim.scalar("ncells")
        stream = torch.cuda.ExternalStream(sim.stream())
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        worst = {"mac_divu_rel": 0.0, "nodal_residual_rel": 0.0, "cell_nodal_divu_rel": 0.0}
        dominant, rep = None, None
        torch.cuda.synchronize()
        for m in range(nsteps):
            # the mixed form's step before the timed window times every kernel (the divergence
            # reads after it are not part of the step); the window times the dominant one
            profiled = form == "mixed" and m == nsteps - args.steps - 1
            if profiled:
                sim.profile_kernels("*")
            ev[m][0].record(stream)
            sim.step()
            ev[m][1].record(stream)
            if profiled:
                rep = sim.profile_report()
                dominant = max((k for k in rep if not k.startswith("(mg_")), key=lambda k: rep[k][1])
                sim.profile_kernels("")
            d = divergence(sim)
            if profiled:
                sim.profile_kernels(dominant)
            for k in worst:
                worst[k] = max(worst[k], d[k])
        torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in ev]
        out = {"ms_all": sum(ms), "ms_last": sum(ms[-args.steps:]), "divergence_max_over_steps": worst, "divergence_final": divergence(sim),
               "fields": {f: sim.get_field(f) for f in ("velocity", "p", "gp")}, "cells": cells}
        if form == "mixed":
            dom = sim.profile_report().get(dominant, (0, 0.0, 0.0))
            sim.profile_kernels("")
            n_l, ms_l, by_l = dom
            achieved = (by_l / n_l) / ((ms_l / n_l) * 1e-3) / 1e9 if n_l else None
            step_bytes = sum(v[2] for v in rep.values())
            step_ms = sum(v[1] for v in rep.values())
            out["roofline"] = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak if achieved else None, "peak_kind": peak_kind, "launches": n_l,
                               "avg_launch_us": 1e3 * ms_l / n_l if n_l else None,
                               "algorithmic_bytes_per_launch": by_l / n_l if n_l else None,
                               "traffic": ncu_traffic("mixed:" + dominant, by_l / n_l if n_l else None)}
            out["step_roofline"] = {"algorithmic_bytes_per_step": step_bytes,
                                    "achieved_GBs": step_bytes / (out["ms_last"] / args.steps * 1e-3) / 1e9,
                                    "frac": step_bytes / (out["ms_last"] / args.steps * 1e-3) / 1e9 / peak,
                                    "note": "bytes: every kernel launcher's algorithmic bytes over one profiled step, at the "
                                            "precision each pass runs in; time: the timed steps' average"}
            out["kernels"] = {"note": "one profiled step: kernel, launches, ms, share, algorithmic GB/s", "top": kernel_table(rep)}
        res[form] = out
        del sim
    r64, rmx = res["fp64"]["fields"], res["mixed"]["fields"]

    def errs(name):
        a, b = rmx[name], r64[name]
        if name == "p":
            a, b = a - a.mean(), b - b.mean()
        d = np.abs(a - b)
        return {"rel_l2": float(np.sqrt((d ** 2).sum() / (b ** 2).sum())), "rel_linf": float(d.max() / np.abs(b).max())}

    dv = np.abs(rmx["velocity"] - r64["velocity"]).ravel() / np.abs(r64["velocity"]).max()
    q = np.quantile(dv, [0.5, 0.99, 0.999, 0.9999])
    cells = res["fp64"]["cells"]
    mx = res["mixed"]
    return {"value": replica_throughput(cells, args.steps, world, mx["ms_last"] * 1e-3), "unit": UNIT,
            "ms_per_step": mx["ms_last"] / args.steps,
            "speedup_vs_fp64": res["fp64"]["ms_last"] / mx["ms_last"],
            "speedup_vs_fp64_all_steps": res["fp64"]["ms_all"] / mx["ms_all"],
            "speedup_vs_fp64_main_run": fp64_ms_main / (mx["ms_last"] / args.steps),
            "steps_compared": nsteps, "timed_window": "last %d of %d steps" % (args.steps, nsteps),
            "errors_vs_fp64": {"velocity": errs("velocity"), "p": errs("p"), "gp": errs("gp"),
                               "velocity_pointwise_rel_quantiles": {"p50": float(q[0]), "p99": float(q[1]), "p99.9": float(q[2]),
                                                                    "p99.99": float(q[3]), "max": float(dv.max())},
                               "velocity_points_above_1e-6": int((dv > 1e-6).sum()), "velocity_points": int(dv.size)},
            "divergence": {"fp64": res["fp64"]["divergence_max_over_steps"], "mixed": mx["divergence_max_over_steps"],
                           "note": "largest value over all steps; mac_divu_rel = max|div u_mac| min(dx) / max|u_mac| after the "
                                   "(exact) MAC projection; nodal_residual_rel = the nodal solve's final / initial residual; "
                                   "cell_nodal_divu_rel = the nodal divergence of the cell velocity after the (approximate) "
                                   "nodal projection, truncation-sized in both forms"},
            "roofline": mx["roofline"], "step_roofline": mx["step_roofline"], "kernels": mx["kernels"],
            "note": "FP32 advection and multigrid cycles, FP64 residuals / defect correction / RHS / velocity update"}


def variant_bench(args, torch, ks, deck, workload, world, rank, label):
    """Another form of the ABL workload (scheme or diffusion treatment): device
    time of --steps steps after --warmup, FP64, with the per-step V-cycle counts."""
    sim = ks.Incflo(deck)
    sim.InitData()
    cells = sim.scalar("ncells")
    for w in range(args.warmup):
        if args.profile_all and w == args.warmup - 1:
            sim.profile_kernels("*")
        sim.step()
    if args.profile_all and rank == 0:
        rep = sim.profile_report()
        tot = sum(v[1] for v in rep.values())
        sys.stderr.write("-- %s step --\n" % label)
        for k, v in sorted(rep.items(), key=lambda kv: -kv[1][1]):
            sys.stderr.write("%-22s %6d launches %9.3f ms %5.1f%% %8.1f GB/s\n" % (k, v[0], v[1], 100 * v[1] / tot,
                                                                                  v[2] / (v[1] * 1e-3) / 1e9 if v[1] else 0))
    sim.profile_kernels("")
    stream = torch.cuda.ExternalStream(sim.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mac_it, nod_it, dif_it = [], [], []
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        sim.step()
        mac_it.append(sim.scalar("mac_iters"))
        nod_it.append(sim.scalar("nodal_iters"))
        dif_it.append(sim.scalar("diff_iters"))
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    out = {"workload": workload, "value": replica_throughput(cells, args.steps, world, ms * 1e-3), "unit": UNIT,
           "ms_per_step": ms / args.steps, "dt": sim.scalar("dt"), "mac_vcycles_per_step": statistics.mean(mac_it),
           "nodal_vcycles_per_step": statistics.mean(nod_it), "diffusion_vcycles_per_solve": statistics.mean(dif_it),
           "divergence": divergence(sim)}
    del sim
    return out


def semi_bench(args, torch, ks, decks, nx, ny, nz, world, rank):
    """The workload with mac_proj.do_semicoarsening = true, the reference's MLMG
    option for cells finer in one direction: the MAC hierarchy halves z alone
    (20 x 20 x 10 m -> 20 x 20 x 20 m cells), then all three directions.  FP64
    and mixed precision, --steps steps after --warmup each.  A failure is
    reported in the line instead of raised."""
    out = {}
    for form in ("fp64", "mixed"):
        deck = (decks.abl(nx, ny, nz, steps=10 ** 9, dz=args.dz) + "\nmac_proj.do_semicoarsening = true\n" +
                ("ks.precision = mixed\n" if form == "mixed" else ""))
        try:
            out[form] = variant_bench(args, torch, ks, deck, "ABL %dx%dx%d, MAC semicoarsening, %s" % (nx, ny, nz, form), world, rank,
                                      "semicoarsened MAC, " + form)
        except Exception as e:  # reported, never silently replaced
            out[form] = {"failed": str(e)[:300]}
            break
    return out


def mol_bench(args, torch, ks, decks, nx, ny, nz, world, rank):
    """The ABL workload advanced with the MOL predictor-corrector
    (incflo.use_godunov = false, explicit diffusion) at CFL 0.45 (MOL requires
    <= 0.5): two MAC and two nodal projections per step."""
    out = variant_bench(args, torch, ks, decks.mol(decks.abl(nx, ny, nz, steps=10 ** 9, cfl=0.45, dz=args.dz)),
                        "ABL %dx%dx%d, MOL predictor-corrector, explicit diffusion, CFL 0.45, FP64" % (nx, ny, nz), world, rank, "MOL")
    out["projections_per_step"] = {"mac": 2, "nodal": 2}
    return out


def cn_bench(args, torch, ks, decks, nx, ny, nz, world, rank):
    """The ABL workload with the reference's default diffusion treatment,
    Crank-Nicolson (incflo.diffusion_type = 1): predictor_rhs with half the old
    diffusion term and a multigrid solve of rho u - dt/2 divtau(u) per step; no
    diffusion CFL."""
    d = decks.abl(nx, ny, nz, steps=10 ** 9, dz=args.dz).replace("incflo.diffusion_type = 0", "incflo.diffusion_type = 1")
    return variant_bench(args, torch, ks, d, "ABL %dx%dx%d, Godunov, Crank-Nicolson diffusion, CFL 0.9, FP64" % (nx, ny, nz), world, rank,
                         "Crank-Nicolson")


def stratified_bench(args, torch, ks, decks, nx, ny, nz, world, rank):
    """The reference's stratified ABL configuration (abl_godunov: temperature
    transport, Boussinesq buoyancy, Coriolis, ABLForcing, heat-flux wall model,
    Crank-Nicolson diffusion of velocity and temperature) on the ABL grid:
    20 m cells, the 3 K/km gradient continued to the top."""
    d = decks.abl_temperature((nx, ny, nz), steps=10 ** 9, diffusion_type=1, fixed_dt=-0.5, size=(20.0 * nx, 20.0 * ny, 20.0 * nz),
                              heights=(650.0, 750.0, 20.0 * nz), values=(300.0, 308.0, 308.0 + 0.003 * (20.0 * nz - 750.0)))
    out = variant_bench(args, torch, ks, d, "stratified ABL %dx%dx%d (20 m cells), temperature + Boussinesq + ABLForcing, Crank-Nicolson, CFL 0.95, "
                        "FP64" % (nx, ny, nz), world, rank, "stratified ABL")
    return out


def adjoint_bench(args, torch, ks, decks):
    """Reverse mode on the adjoint-check workload: 128 x 128 x 64 periodic box,
    3 uniform-Ct disks, J = wake-box kinetic energy after 40 steps.  Device
    time (CUDA events on the handle's stream) of forward steps, of reverse
    steps (each recomputes its forward step in FP64) and of a whole
    checkpointed run; dJ/dCt against central finite differences."""
    nsteps, slots = 40, 6  # binomial schedule; the store-every-state run uses nsteps slots
    deck, lo, hi, cts = decks.adjoint_c3()
    sim = ks.Incflo(deck)
    sim.InitData()
    sim.set_objective_box(lo, hi)
    x0 = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    ct = [float(c) for c in cts]
    stream = torch.cuda.ExternalStream(sim.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def restore():
        for f, v in x0.items():
            sim.set_field(f, v)
        sim.set_disk_ct(ct)

    def timed(fn, k):
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    for _ in range(args.warmup):
        sim.step()
    fwd = timed(sim.step, args.steps) / args.steps
    sim.adjoint_reset()
    sim.objective(seed=True)
    for _ in range(args.warmup):
        sim.adjoint_step()
    rev = timed(sim.adjoint_step, args.steps) / args.steps
    restore()
    J = [None]

    def run():
        J[0] = sim.adjoint_run(nsteps, slots)

    run_ms = timed(run, 1)
    g = sim.ct_gradient()
    added = sim.scalar("adj_forward_steps")
    restore()
    J_all = [None]

    def run_all():
        J_all[0] = sim.adjoint_run(nsteps, nsteps)

    all_ms = timed(run_all, 1)
    g_all = sim.ct_gradient()
    added_all = sim.scalar("adj_forward_steps")
    free, total = torch.cuda.mem_get_info()

    def fJ(c):
        for f, v in x0.items():
            sim.set_field(f, v)
        sim.set_disk_ct(c)
        for _ in range(nsteps):
            sim.step()
        return sim.objective()

    fd = {}
    for h in (1e-8, 1e-6):
        est = []
        for k in range(len(ct)):
            cp = list(ct)
            cm = list(ct)
            cp[k] += h
            cm[k] -= h
            est.append((fJ(cp) - fJ(cm)) / (2 * h))
        fd["%g" % h] = max(abs(a - b) for a, b in zip(est, g)) / max(abs(x) for x in g)
    return {"workload": "128x128x64 periodic, 8 m/s + 0.2 m/s noise, 3 UniformCt disks (D = 16 cells), laminar, dt = 1 s, "
                        "J = mean 0.5|u|^2 in the wake box after %d steps" % nsteps,
            "forward_ms_per_step": fwd, "adjoint_ms_per_step": rev, "adjoint_over_forward_step": rev / fwd,
            "checkpointed_run": {"steps": nsteps, "snapshots": slots, "forward_steps_added": added, "ms": run_ms,
                                 "over_forward_run": run_ms / (nsteps * fwd)},
            "store_all_run": {"steps": nsteps, "snapshots": nsteps, "forward_steps_added": added_all, "ms": all_ms,
                              "over_forward_run": all_ms / (nsteps * fwd),
                              "grad_rel_diff_vs_checkpointed": max(abs(a - b) for a, b in zip(g, g_all)) / max(abs(x) for x in g)},
            "J": J[0], "dJ_dCt": list(g), "Ct": ct,
            "fd_rel_err": {"h=1e-8": fd["1e-08"], "h=1e-6": fd["1e-06"],
                           "note": "the discrete map has jumps (PPM limiter / trace-switch / Riemann branches) about 1e-7 "
                                   "apart in Ct: h = 1e-6 sums dozens of them, h = 1e-8 mostly stays on one smooth piece"},
            "device_mem_in_use_GB": (total - free) / 1e9}


def c4_bench(args):
    """Production forward + adjoint run: 512x512x256 ABL (C1 physics at 10 m
    cells, 5120x5120x2560 m) with a 4x4 farm of uniform-Ct
    disks (D = 20 cells, spacing 7 D), fixed dt 0.5 s, mixed-precision forward
    with binomial checkpoints in HBM and the FP64 reverse sweep; dJ/dCt of two
    disks against central finite differences of the FP64 forward."""
    import torch
    import kynema_sgf_gb300 as ks
    from kynema_sgf_gb300 import decks
    nsteps, slots = args.c4_steps, args.c4_slots
    deck, lo, hi, cts = decks.abl_disks()
    sim = ks.Incflo(deck)
    sim.InitData()
    sim.set_objective_box(lo, hi)
    dev = torch.device("cuda:0")
    x0 = {f: torch.empty(sim.layout(f), dtype=torch.float64, device=dev) for f in ("velocity", "gp", "p")}
    for f, t in x0.items():
        sim.get_field(f, out=t)
    stream = torch.cuda.ExternalStream(sim.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def restore(c=cts):
        for f, t in x0.items():
            sim.set_field(f, t)
        sim.set_disk_ct(c)

    def timed(fn, k):
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    restore()
    sim.step()
    fwd_mixed = timed(sim.step, 3) / 3
    restore()
    sim.set_precision(0)
    fwd64 = timed(sim.step, 3) / 3
    sim.set_precision(1)
    restore()
    sim.adjoint_reset()
    sim.objective(seed=True)
    sim.adjoint_step()
    rev = timed(sim.adjoint_step, 2) / 2
    sim.profile_kernels("*")
    sim.adjoint_step()
    rep = sim.profile_report()
    sim.profile_kernels("")
    tot = sum(v[1] for v in rep.values())
    top = [[k, v[0], round(v[1], 2), round(v[1] / tot, 3)] for k, v in sorted(rep.items(), key=lambda kv: -kv[1][1])[:16]]
    restore()
    out = {}

    def run():
        out["J"] = sim.adjoint_run(nsteps, slots)

    run_ms = timed(run, 1)
    g = [float(x) for x in sim.ct_gradient()]
    added = sim.scalar("adj_forward_steps")
    free, total = torch.cuda.mem_get_info()
    lib_mem = (total - free) - torch.cuda.memory_reserved()
    sim.set_precision(0)
    # the same checkpointed run on the FP64 forward: separates the effect of
    # the mixed-precision trajectory from finite-difference error
    restore()
    out64 = {}

    def run64():
        out64["J"] = sim.adjoint_run(nsteps, slots)

    run64_ms = timed(run64, 1)
    g64 = [float(x) for x in sim.ct_gradient()]

    def fJ(c):
        restore(c)
        for _ in range(nsteps):
            sim.step()
        return sim.objective()

    J64 = fJ(cts)
    fd = {}
    for h in (float(x) for x in args.c4_fd_h.split(",") if x):
        est, fwd, bwd = [], [], []
        for k in (0, 1):
            cp, cm = list(cts), list(cts)
            cp[k] += h
            cm[k] -= h
            Jp, Jm = fJ(cp), fJ(cm)
            est.append((Jp - Jm) / (2 * h))
            fwd.append((Jp - J64) / h)  # one-sided slopes: they differ where a jump of the discrete map lies within h
            bwd.append((J64 - Jm) / h)
        gm = max(abs(x) for x in g[:2])
        fd["h=%g" % h] = {"fd": est, "rel_err_mixed_adjoint": [abs(a - b) / gm for a, b in zip(est, g[:2])],
                          "rel_err_fp64_adjoint": [abs(a - b) / gm for a, b in zip(est, g64[:2])],
                          "one_sided_fp64_adjoint_rel_err": [[abs(a - c) / gm, abs(b - c) / gm] for a, b, c in zip(fwd, bwd, g64[:2])],
                          "J_rounding_as_slope_rel": float(np.spacing(J64)) / h / gm}
    line = {"c4": {
        "workload": "512x512x256 ABL (C1 physics, 10 m cells), 4x4 UniformCt disks D = 20 cells spaced 7 D, fixed dt 0.5 s, "
                    "J = mean 0.5|u|^2 in the rotor layer 0..5 D behind the first column, %d steps" % nsteps,
        "forward_mixed_ms_per_step": fwd_mixed, "forward_fp64_ms_per_step": fwd64,
        "reverse_step_ms": rev, "reverse_step_over_mixed_forward": rev / fwd_mixed,
        "reverse_step_kernels": {"note": "one reverse step (with its recompute), kernel, launches, ms, share", "top": top},
        "run": {"steps": nsteps, "snapshots": slots, "forward_steps_added": added, "ms": run_ms,
                "over_mixed_forward_run": run_ms / (nsteps * fwd_mixed)},
        "device_mem_library_GB": lib_mem / 1e9, "device_mem_in_use_GB": (total - free) / 1e9,
        "J_mixed_forward": out["J"], "J_fp64_forward": J64, "dJ_dCt": g,
        "fp64_run": {"ms": run64_ms, "J": out64["J"], "dJ_dCt": g64,
                     "rel_diff_mixed_vs_fp64_adjoint": max(abs(a - b) for a, b in zip(g, g64)) / max(abs(x) for x in g64)},
        "fd_fp64_disks_0_1": fd}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.c4:
        c4_bench(args)
        return
    if args.cpu_worker:
        cpu_worker(args.cpu_worker)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        # the full workload (not a sample): Evolve steps of the 256x256x128 deck on all host cores, as
        # many of --steps as fit in --ref-budget seconds (a warm-up cut short after a quarter of it)
        size = tuple(int(x) for x in args.size.split(","))
        cells, rates, runs, cores = run_cpu(args.warmup, args.steps, 1, size, dz=args.dz, budget=args.ref_budget)
        per = runs[0]
        v = rates[0]
        what = ("CPU restatement (oracle/ks_oracle.cpp, g++ -O3 -fopenmp; the reference's own build cannot be compiled: its "
                "AMReX / AMReX-Hydro submodules are absent) on the full %dx%dx%d workload, %d timed Evolve steps of the %d asked "
                "(budget %g s) after up to %d untimed, initialisation skipped" % (size + (len(per), args.steps, args.ref_budget,
                                                                                  args.warmup)))
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "steps_timed": len(per),
                "warmup": args.warmup, "ms_per_step": 1e3 * sum(per) / len(per), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": DATA, "config": workload_config(size, args.dz, world),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": what, "cpu": cpu_model()},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
    r = our_arm(args, rank, world, local_rank)
    if rank != 0:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()
        return
    peak, peak_kind = peaks()
    n_l, ms_l, by_l = r["dom"]
    achieved = (by_l / n_l) / ((ms_l / n_l) * 1e-3) / 1e9 if n_l else None
    traffic = ncu_traffic(r["dominant"], by_l / n_l if n_l else None)
    nx, ny, nz = r["size"]
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA, "config": workload_config((nx, ny, nz), args.dz, world),
            "solver": {"mac_vcycles_per_step": r["mac"], "nodal_vcycles_per_step": r["nodal"]},
            "divergence": r["div"],
            "roofline": {"bound": "hbm", "kernel": r["dominant"], "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic, "peak_kind": peak_kind,
                         "launches": n_l, "avg_launch_us": 1e3 * ms_l / n_l if n_l else None,
                         "algorithmic_bytes_per_launch": by_l / n_l if n_l else None},
            "gpu_launches": r["launches"], "clocks": r["clocks"], "e2e": r["e2e"], "mixed_precision": r["mixed"],
            "adjoint": r["adjoint"], "tgv64": r["tgv"], "mol": r["mol"], "crank_nicolson": r["cn"],
            "stratified_abl": r["strat"], "mac_semicoarsening": r["semi"]}
    # The FP64 path is bound by FP64 issue on this GPU (the nodal sweep's FP64 pipe is 81-83 % busy
    # under ncu): report the dominant kernel against the FMA peak measured live by ks_fma_peak as well.
    fl = FP64_FLOPS_PER_BYTE.get(r["dominant"])
    if fl and achieved:
        line["fp64_roofline"] = {"kernel": r["dominant"], "achieved_gflops": achieved * fl, "peak_gflops": r["fp64_peak"],
                                 "frac": achieved * fl / r["fp64_peak"], "peak_kind": "measured live (ks_fma_peak, FP64 FMA chains)",
                                 "flops_per_unit": "FP64 flops per unit as in FP64_FLOPS_PER_BYTE (an FMA counts 2)"}
    # whole-step algorithmic traffic: 8 * (125 + 20.86 * V-cycles) bytes per cell
    bstep = 8.0 * (125.0 + 20.86 * (r["mac"] + r["nodal"])) * r["cells"]
    line["step_roofline"] = {"algorithmic_bytes_per_step": bstep, "achieved_GBs": bstep / (r["ms"] / args.steps * 1e-3) / 1e9,
                             "frac": bstep / (r["ms"] / args.steps * 1e-3) / 1e9 / peak}
    if world == 1 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline_entry(1, 5, 5, dz=args.dz)
        except Exception as e:  # reported, never silently replaced
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": "failed: %s" % e}
        try:
            r["tgv"]["cpu"] = cpu_baseline_entry(1, 5, 3, case="tgv", what="CPU restatement, the same 64^3 Taylor-Green deck")
        except Exception as e:
            r["tgv"]["cpu"] = {"value": None, "sample": "failed: %s" % e}
        if r["mol"]:
            try:
                r["mol"]["cpu"] = cpu_baseline_entry(1, 3, 3, case="mol", what="CPU restatement, MOL form of the %dx%dx%d ABL sample"
                                                     % CPU_SAMPLE, dz=args.dz)
            except Exception as e:
                r["mol"]["cpu"] = {"value": None, "sample": "failed: %s" % e}
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
