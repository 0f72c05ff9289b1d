"""Benchmark of the docking energy+gradient hot path on one GB300.

Default workload: rigid scoring at scale (receptor 2,000 beads, ligand 700
beads, 100,000 seeded random poses on a 40-55 A shell, 0.9/1.8 A grids with 33
float4 channels, 10 A plateau), one fused energy+gradient launch per step;
metric = energy+gradient evaluations per second.

  value    device-resident throughput: poses / kernel time (CUDA events on the
           launching stream), L2 flushed (256 MB write) between steps
  e2e      the same metric through the public C ABI with pinned HOST buffers:
           H2D of the poses, the launch, D2H of the results, every step
  roofline algorithmic bytes per launch (census: 52 B per pose + 128 B per
           grid-channel octet + 8 B per NL voxel lookup + 4 B per list entry)
           / kernel time, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a C++ port of the reference CPU path) on a
           bounded sample of the same workload, all host threads

`--impl reference` times the reference's CPU implementation of the path (the
port, or the reference build in oracle/_ref where it exists) on the same
workload and prints one line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "E+grad evals/s"
UNIT = "evals/s"
WORKLOAD = "rigid scoring, receptor 2000 / ligand 700 beads, 100000 poses (config 1)"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path("/tmp") / f"gba_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_workload(n_poses: int | None):
    import __graft_entry__
    pkg = __graft_entry__.load_package()
    wl = pkg.synth.make_config(1, n_poses=n_poses)
    return pkg, wl


def cpu_rate(pkg, wl, grid_host, seconds: float, nthreads: int):
    """Oracle-port evals/s on a bounded sample of the workload's poses."""
    from oracle import pyoracle as po
    probe = wl.dofs[:64]
    t0 = time.perf_counter()
    po.energy_6d(wl.rec, wl.lig, grid_host, wl.params, probe, nthreads=nthreads)
    dt = max(time.perf_counter() - t0, 1e-4)
    n = int(min(len(wl.dofs), max(64, 64 * seconds / dt)))
    sample = wl.dofs[:n]
    t0 = time.perf_counter()
    po.energy_6d(wl.rec, wl.lig, grid_host, wl.params, sample, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    from oracle import pyoracle as po
    pkg, wl = make_workload(args.poses)
    nthreads = os.cpu_count() or 1
    grid = po.build_grid(wl.rec, wl.params, pkg.GridOptions(), nthreads=nthreads)
    kind = "reference" if po.ref_available() else "port"
    per_step = int(args.ref_sample)
    rates = []
    for s in range(args.warmup + args.steps):
        off = (s * per_step) % max(1, len(wl.dofs) - per_step)
        sample = wl.dofs[off: off + per_step]
        t0 = time.perf_counter()
        if kind == "reference":
            po.ref_energy_6d(wl.rec, wl.lig, grid, wl.params, sample, nworkers=nthreads, item_size=1000)
        else:
            po.energy_6d(wl.rec, wl.lig, grid, wl.params, sample, nthreads=nthreads)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            rates.append(per_step / dt)
    value = float(len(rates) * per_step / sum(per_step / r for r in rates))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * per_step / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "poses_per_step": per_step},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind,
                             "sample": f"{per_step} poses of the workload per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbattract", choices=["gbattract", "reference"])
    ap.add_argument("--poses", type=int, default=None, help="override the pose count")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-sample", type=int, default=2000)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import __graft_entry__
    pkg, wl = make_workload(args.poses)
    from gbattract.context import GbaContext
    ctx = GbaContext(local)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    t0 = time.perf_counter()
    grid = ctx.build_grid(rec, par, pkg.GridOptions())
    torch.cuda.synchronize()
    log(f"grid build {time.perf_counter() - t0:.2f}s")
    n = len(wl.dofs)
    dofs = torch.from_numpy(wl.dofs).cuda()
    out = torch.empty((n, 7), dtype=torch.float32, device="cuda")
    # census (outside the timed region): algorithmic bytes per launch
    cen, _ = ctx.census_6d(rec, lig, grid, par, dofs)
    cen = cen.cpu().numpy().astype(np.int64)
    bytes_launch = int(52 * n + 128 * (cen[:, 0].sum() + cen[:, 1].sum()) + 8 * cen[:, 2].sum() +
                       4 * cen[:, 3].sum())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        ctx.energy_6d(rec, lig, grid, par, dofs, out=out, stream=sptr)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            times.append((e0, e1))
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        if world > 1:
            torch.distributed.barrier()
    ks = [a.elapsed_time(b) / 1000.0 for a, b in times]
    ktot = sum(ks)
    if world > 1:
        t = torch.tensor([ktot], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ktot = float(t.item())
    value = world * n * args.steps / ktot
    kavg = ktot / args.steps
    achieved = bytes_launch / kavg / 1e9
    peak, peak_kind = measured_peaks()

    # end to end through the C ABI with pinned host buffers
    hd = torch.from_numpy(wl.dofs).pin_memory()
    ho = torch.empty((n, 7), dtype=torch.float32).pin_memory()
    for _ in range(2):
        ctx.energy_6d(rec, lig, grid, par, hd, out=ho)
    torch.cuda.synchronize()
    e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e_steps):
        ctx.energy_6d(rec, lig, grid, par, hd, out=ho)
    e2e_dt = (time.perf_counter() - t0) / e_steps
    e2e = world * n / e2e_dt

    # parity spot check of the timed result (device path) against the host path
    ok = bool(np.array_equal(out.cpu().numpy(), ho.numpy()))

    cpu = None
    if rank == 0 and not args.no_cpu:
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
        gh = ctx.download_grid(grid)
        nthreads = os.cpu_count() or 1
        rate, ns, dt = cpu_rate(pkg, wl, gh, args.cpu_seconds, nthreads)
        cpu = {"value": rate, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"first {ns} poses of the workload ({dt:.1f} s on {nthreads} threads)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * kavg, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "poses": n, "receptor_beads": wl.rec.n,
                       "ligand_beads": wl.lig.n, "l2": "flushed (256 MB write) between steps",
                       "grid_MB": None},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(24 * n),
                    "d2h_bytes_per_step": int(28 * n)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                         "bytes_per_launch": bytes_launch},
            "cpu_baseline": cpu, "clocks": clk.summary(), "gpu_launches": args.steps,
            "wall_s_timed": wall, "host_device_paths_equal": ok,
            "census": {"grid_lookups_per_pose": float(cen[:, 0].mean()),
                       "charged_per_pose": float(cen[:, 1].mean()),
                       "nl_beads_per_pose": float(cen[:, 2].mean()),
                       "nl_entries_per_pose": float(cen[:, 3].mean())},
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
