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
           grid-channel octet + 8 B per NL voxel lookup + 24 B per list entry:
           index, receptor xyz, type, charge) / energy-kernel time (CUDA events
           the library records around the launch), against the measured HBM
           copy bandwidth
           (plus the same achieved figure against an L2 copy bandwidth measured
           in the run: "roofline.l2")
  cpu_baseline  the CPU oracle (a C++ port of the reference CPU path) on a
           bounded sample of the same workload, all host threads
  parity   the timed workload's own GPU results on the first 20,000 poses
           against the oracle (FP32, FP64, correctly rounded sin/cos)
  minimization   config 0 (1,000 poses, maxFunEval 100): device-resident
           batched form vs the plain per-step forms and the CPU oracle
  batched_uneven config 4 (64 pairs, 1.65 M poses, maxFunEval 500): one
           persistent work-queue launch in a CUDA graph with default and with
           autotuned per-pair shapes, vs the plain per-step form on every 8th
           pair, per-pair completion times, oracle agreement on a sample
  suite    config 2 (normal modes: scoring with its census roofline, device
           vs plain minimization) and config 3 (pairwise energy and adjoint)

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
KOPT_REFERENCE_ORDER = 16    # GBA_KOPT_REFERENCE_ORDER: the reference CPU path's summation order


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
                 "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
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


def traffic_per_pose(variant: str):
    """DRAM bytes per pose of the energy kernel from profiles/traffic.json
    (one ncu capture of the same kernel and variant, with its command), or
    None for another variant."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None, None
    d = json.loads(p.read_text()).get("rigid_energy_kernel", {})
    if d.get("variant") != variant:
        return None, None
    return float(d["dram_bytes_per_pose"]), "profiles/traffic.json (" + d.get("summary", "") + ")"


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def shard(dofs, world: int, rank: int):
    """Rank `rank`'s share of a job of `world` equal contiguous pose slices
    (weak scaling: each rank scores its own poses, no collective on the data
    path)."""
    n = len(dofs) // world
    return dofs[rank * n:(rank + 1) * n]


def max_over_ranks(values, world: int, device: str = "cuda"):
    """Element-wise maximum of a list of floats over all ranks (the slowest
    rank sets a step's time); identity for one rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def make_workload(n_poses: int | None, rec_beads: int | None = None):
    """Config 1 (or, for small profiling captures, config 1's distributions with
    a smaller receptor)."""
    import __graft_entry__
    pkg = __graft_entry__.load_package()
    if rec_beads:
        c = pkg.synth.CONFIGS[1]
        wl = pkg.synth.make_pair(1, rec_beads, c["lig"], n_poses or c["poses"], c["shell"])
    else:
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


def timed_result_parity(wl, grid_host, got, m: int, nthreads: int, ro=None):
    """Parity of the timed workload's own GPU results (the first m poses)
    against the CPU oracle on the same, device-built grid: the scaled error
    bound of the tests, the share of poses within 1e-4 of the bare relative
    error, the errors of the GPU and of the FP32 oracle against the FP64
    oracle; and the same against the oracle with correctly rounded sin/cos
    (the C library's sinf/cosf misround a few percent of angles by one ulp).
    ro: the same batch scored in the reference's summation order, compared
    bit for bit with both oracles."""
    from oracle import pyoracle as po
    d = wl.dofs[:m]
    ref, st = po.energy_6d(wl.rec, wl.lig, grid_host, wl.params, d, stats=True, nthreads=nthreads)
    ref64 = po.energy_6d_f64(wl.rec, wl.lig, grid_host, wl.params, d, nthreads=nthreads)
    with po.exact_sincos():
        ref_x = po.energy_6d(wl.rec, wl.lig, grid_host, wl.params, d, nthreads=nthreads)
    exact = po.libm_sincos_rounds_exactly(d[:, 3:6])
    out = po.parity_stats(got[:m], ref, st, ref64)
    out["poses_with_correctly_rounded_libm_sincos"] = int(exact.sum())
    out["max_scaled_err_those_poses"] = po.parity_stats(got[:m][exact], ref[exact], st[exact])["max_scaled_err"]
    vs_x = po.parity_stats(got[:m], ref_x, st)
    out["vs_correctly_rounded_sincos_oracle"] = {k: vs_x[k] for k in ("max_scaled_err", "frac_within_1e-4_bare")}
    if ro is not None:
        same = np.all(ro[:m] == ref_x, axis=1)
        out["reference_order"] = {
            "bitwise_equal_correctly_rounded_sincos_oracle": bool(same.all()),
            "poses_bitwise_equal_oracle": int(np.all(ro[:m] == ref, axis=1).sum()),
            "poses_bitwise_equal_oracle_of_those_with_correctly_rounded_libm_sincos":
                int(np.all(ro[:m][exact] == ref[exact], axis=1).sum())}
    out["bound"] = "per pose |d| / max(|ref|, 0.05 S) <= 1e-4 for E, force and torque, S = sum of |terms|"
    return out


def measured_l2_peak(device: str = "cuda"):
    """Copy bandwidth of a 2 x 48 MB working set, resident in the 129 MB L2:
    50 back-to-back copies replayed from a CUDA graph (no launch gaps), best
    of 5 replays (read + write bytes)."""
    import torch
    n = 48 * 1024 * 1024 // 4
    a = torch.ones(n, dtype=torch.float32, device=device)
    b = torch.empty_like(a)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            b.copy_(a)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(50):
            b.copy_(a)
    g.replay()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1000.0)
    return 50 * 2 * a.numel() * 4 / best / 1e9


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    from oracle import pyoracle as po
    pkg, wl = make_workload(args.poses, args.rec_beads)
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


def bench_minimization(ctx, pkg, nthreads: int, with_cpu: bool, kopts: int = 15):
    """Config 0 (receptor 500 / ligand 200 beads, 1000 poses, 100-evaluation VA13):
    minimized poses/s of the device-resident batched form, of the plain per-step
    forms (one launch per round; the reference's 100-pose work items) and of the
    CPU oracle's VA13 on all host threads, with the agreement of the minimized
    energies; and the batched form in the reference's summation order
    (GBA_KOPT_REFERENCE_ORDER), its cost and its bitwise equality with the
    oracle taking correctly rounded sin/cos -- and, with the host C library's
    sin/cos tabulated (gba_set_host_sincos), with the oracle as the reference
    runs it."""
    import torch
    wl = pkg.synth.make_config(0)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    grid = ctx.build_grid(rec, par, pkg.GridOptions())
    ids = (rec, lig, grid, par)
    n, steps = len(wl.dofs), wl.steps
    ctx.minimize_6d(*ids, wl.dofs[:128], max_evals=steps)          # warm-up, graph capture
    ctx.minimize_6d(*ids, wl.dofs, max_evals=steps)
    torch.cuda.synchronize()
    # a run takes a few ms: the median of five
    runs = []
    for _ in range(5):
        t0 = time.perf_counter()
        s_dev, r_dev, n_dev = ctx.minimize_6d(*ids, wl.dofs, max_evals=steps)
        runs.append(time.perf_counter() - t0)
    dt_dev = float(np.median(runs))
    out = {"workload": f"config 0: receptor {wl.rec.n} / ligand {wl.lig.n} beads, {n} poses, "
                       f"maxFunEval {steps}",
           "batched_device_poses_per_s": n / dt_dev, "batched_device_s": dt_dev,
           "evals_per_pose_mean": float(n_dev.mean())}
    # roofline of the batched form: the census bytes of an evaluation (taken
    # at the start poses) times the evaluations made, plus the VA13 state
    # traffic, over the wall time -- latency-bound by the VA13 steps' FP64
    # chains, not by memory
    cen, _ = ctx.census_6d(*ids, wl.dofs)
    cen = np.asarray(cen.cpu().numpy() if hasattr(cen, "cpu") else cen, np.int64)
    b_eval = 52 + 128 * (cen[:, 0].mean() + cen[:, 1].mean()) + 8 * cen[:, 2].mean() + 24 * cen[:, 3].mean()
    state = 8 * (6 + 21 + 6 * 7)
    achieved = (b_eval + state) * float(n_dev.sum()) / dt_dev / 1e9
    peak, kind = measured_peaks()
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "peak_source": kind, "bytes_per_eval": b_eval, "state_bytes_per_step": state,
                       "evals": int(n_dev.sum())}
    for item, key in ((0, "plain_one_launch_per_round"), (100, "plain_100_pose_items")):
        ctx.minimize_6d_plain(*ids, wl.dofs[:64], max_evals=10, item_size=item)
        t0 = time.perf_counter()
        s_p, r_p, n_p = ctx.minimize_6d_plain(*ids, wl.dofs, max_evals=steps, item_size=item)
        dt = time.perf_counter() - t0
        out[key + "_poses_per_s"] = n / dt
        out[key + "_identical_to_batched"] = bool(np.array_equal(r_p, r_dev))
    ctx.set_kernel_options(kopts | KOPT_REFERENCE_ORDER)
    ctx.minimize_6d(*ids, wl.dofs[:128], max_evals=steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ro = ctx.minimize_6d(*ids, wl.dofs, max_evals=steps)
    dt_ro = time.perf_counter() - t0
    # and with the host C library's sin/cos: the reference's values on this host
    t0 = time.perf_counter()
    ctx.set_host_sincos(4096.0)
    out["host_sincos_table_s"] = time.perf_counter() - t0
    ctx.minimize_6d(*ids, wl.dofs[:128], max_evals=steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rh = ctx.minimize_6d(*ids, wl.dofs, max_evals=steps)
    dt_rh = time.perf_counter() - t0
    ctx.set_host_sincos(0)
    ctx.set_kernel_options(kopts)
    out["reference_order_host_sincos_poses_per_s"] = n / dt_rh
    out["reference_order_poses_per_s"] = n / dt_ro
    out["reference_order_time_ratio"] = dt_ro / dt_dev
    out["speedup_vs_plain_one_launch"] = out["batched_device_poses_per_s"] / out["plain_one_launch_per_round_poses_per_s"]
    out["speedup_vs_plain_100_pose_items"] = out["batched_device_poses_per_s"] / out["plain_100_pose_items_poses_per_s"]
    if with_cpu:
        from oracle import pyoracle as po
        gh = ctx.download_grid(grid)
        t0 = time.perf_counter()
        s_cpu, r_cpu, n_cpu = po.minimize_6d(wl.rec, wl.lig, gh, wl.params, wl.dofs, steps, nthreads=nthreads)
        dt = time.perf_counter() - t0
        rel = np.abs(r_dev[:, 0].astype(np.float64) - r_cpu[:, 0]) / np.maximum(np.abs(r_cpu[:, 0]), 1e-3)
        out["cpu_oracle_poses_per_s"] = n / dt
        out["cpu_cores"] = nthreads
        out["agreement_within_1e-3"] = float(np.mean(rel <= 1e-3))
        # the reference minimizer's own sensitivity: the oracle against itself
        # with every start pose moved by one ulp in x
        d1 = wl.dofs.copy()
        d1[:, 0] = np.nextafter(d1[:, 0], np.float32(np.inf))
        _, r_ulp, _ = po.minimize_6d(wl.rec, wl.lig, gh, wl.params, d1, steps, nthreads=nthreads)
        rel = np.abs(r_ulp[:, 0].astype(np.float64) - r_cpu[:, 0]) / np.maximum(np.abs(r_cpu[:, 0]), 1e-3)
        out["oracle_self_agreement_one_ulp_start"] = float(np.mean(rel <= 1e-3))
        rel = np.abs(ro[1][:, 0].astype(np.float64) - r_cpu[:, 0]) / np.maximum(np.abs(r_cpu[:, 0]), 1e-3)
        out["reference_order_agreement_within_1e-3"] = float(np.mean(rel <= 1e-3))
        rel = np.abs(rh[1][:, 0].astype(np.float64) - r_cpu[:, 0]) / np.maximum(np.abs(r_cpu[:, 0]), 1e-3)
        out["reference_order_host_sincos_agreement_within_1e-3"] = float(np.mean(rel <= 1e-3))
        out["reference_order_host_sincos_bitwise_equal_oracle"] = bool(
            np.array_equal(rh[0], s_cpu) and np.array_equal(rh[1], r_cpu) and np.array_equal(rh[2], n_cpu))
        with po.exact_sincos():
            x = po.minimize_6d(wl.rec, wl.lig, gh, wl.params, wl.dofs, steps, nthreads=nthreads)
        out["reference_order_bitwise_equal_exact_sincos_oracle"] = bool(
            all(np.array_equal(a, b) for a, b in zip(ro, x)))
    for i in (grid, lig, rec, par):
        ctx.release(i)
    return out


def modes_roofline(ctx, wl, gr, gl, n: int, launch_s: float):
    """Algorithmic bytes of the modes kernel from the oracle's per-pose counts
    on a 2,048-pose sample (bit-exact with the kernel's lookups and neighbour
    walks): per evaluation 104 B DOF + 108 B result + 128 B per grid-channel
    lookup of both passes (ligand beads in the receptor grid, receptor beads
    in the ligand grid) + 8 B per NL voxel lookup + (24 + 12 Mr) B per list
    entry (index, receptor xyz, type, charge and the receptor's Mr mode
    vectors, from which the kernel re-deforms the neighbour); per-bead
    constants count once per batch.  Against the measured HBM copy peak."""
    from oracle import pyoracle as po
    m = min(2048, len(wl.dofs))
    hr, hl = ctx.download_grid(gr), ctx.download_grid(gl)
    _, st = po.energy_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, wl.dofs[:m], stats=True)
    Mr = wl.rec.n_modes
    look = (st["n_grid"].astype(np.float64) + st["n_grid_charged"] + st["n_rec_lookups"]).mean()
    per = 104 + 108 + 128 * look + 8 * st["n_nl"].mean() + (24 + 12 * Mr) * st["n_nl_entries"].mean()
    achieved = per * n / launch_s / 1e9
    peak, kind = measured_peaks()
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": kind, "bytes_per_eval": per, "lookups_per_eval": look,
            "nl_entries_per_eval": float(st["n_nl_entries"].mean()), "kernel_ms_avg": 1000.0 * launch_s,
            "census_sample_poses": m}


def bench_modes(ctx, pkg, n_poses: int, steps: int, minimize: bool = True, with_cpu: bool = True,
                small: bool = False, kopts: int = 15):
    """Config 2: receptor 1500 / ligand 600 beads with 5 modes each: modes
    energy+gradient evals/s, and (minimize) device vs plain minimization; the
    scoring in the reference's summation order, and (minimize, with_cpu) a
    64-pose minimization in that order with the host's sin/cos against the
    oracle."""
    import torch
    if small:
        c = pkg.synth.CONFIGS[2]
        wl = pkg.synth.make_pair(2, 700, 300, n_poses, c["shell"], steps=c["steps"], n_modes=c["modes"])
    else:
        wl = pkg.synth.make_config(2, n_poses=n_poses)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    gr = ctx.build_grid(rec, par, pkg.GridOptions())
    gl = ctx.build_grid(lig, par, pkg.GridOptions())
    for g in (gr, gl):
        ctx.grid_octets(g, True)      # cooperative 8-lane lookups in both passes
    ids = (rec, lig, gr, gl, par)
    d = torch.from_numpy(wl.dofs).cuda()
    out = ctx.energy_6d_modes(*ids, d)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        ctx.energy_6d_modes(*ids, d, out=out, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    launch_s = e0.elapsed_time(e1) / 1000.0 / 3
    evals = len(wl.dofs) / launch_s
    ctx.set_kernel_options(kopts | KOPT_REFERENCE_ORDER)
    ro_out = ctx.energy_6d_modes(*ids, d)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx.energy_6d_modes(*ids, d, out=ro_out, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.set_kernel_options(kopts)
    reference_order = {"evals_per_s": len(wl.dofs) / (e0.elapsed_time(e1) / 1000.0),
                       "time_ratio": e0.elapsed_time(e1) / 1000.0 / launch_s}
    del ro_out
    roof = None
    parity = None
    if with_cpu:
        roof = modes_roofline(ctx, wl, gr, gl, len(wl.dofs), launch_s)
        # parity of the scored batch's first 512 poses: FP32 oracle and FP64
        from oracle import pyoracle as po
        hr, hl = ctx.download_grid(gr), ctx.download_grid(gl)
        d512 = np.ascontiguousarray(wl.dofs[:512])
        ref, st = po.energy_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, d512, stats=True)
        ref64 = po.energy_6d_modes_f64(wl.rec, wl.lig, hr, hl, wl.params, d512)
        parity = po.modes_parity_stats(out[:512].cpu().numpy(), ref, st, ref64, wl.rec.n_modes,
                                       wl.lig.n_modes)
    if not minimize:
        for i in (gr, gl, lig, rec, par):
            ctx.release(i)
        return {"workload": f"config 2{' distributions' if small else ''}: receptor {wl.rec.n} / ligand "
                            f"{wl.lig.n} beads, 5+5 modes; {len(wl.dofs)} poses scored", "energy_evals_per_s": evals,
                "roofline": roof, "parity": parity, "reference_order": reference_order}
    sub = wl.dofs
    ctx.minimize_6d_modes(*ids, sub[:64], max_evals=10)
    t0 = time.perf_counter()
    _, r1, n1 = ctx.minimize_6d_modes(*ids, sub, max_evals=steps)
    dt_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, r2, _ = ctx.minimize_6d_modes_plain(*ids, sub, max_evals=steps)
    dt_plain = time.perf_counter() - t0
    e0 = out[: len(sub), 0].cpu().numpy()
    # the reference's execution model (100-pose work items, one launch each)
    # on a 5,000-pose subset, against the device form on the same subset
    few = sub[:5000]
    t0 = time.perf_counter()
    _, r4, _ = ctx.minimize_6d_modes(*ids, few, max_evals=steps)
    dt_dev_few = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, r5, _ = ctx.minimize_6d_modes_plain(*ids, few, max_evals=steps, item_size=100)
    dt_items = time.perf_counter() - t0
    res = {"workload": f"config 2: receptor {wl.rec.n} / ligand {wl.lig.n} beads, 5+5 modes; "
                       f"{len(wl.dofs)} poses scored, {len(sub)} minimized (maxFunEval {steps})",
           "energy_evals_per_s": evals, "roofline": roof, "parity": parity,
           "minimize_device_poses_per_s": len(sub) / dt_dev,
           "minimize_plain_poses_per_s": len(sub) / dt_plain, "speedup": dt_plain / dt_dev,
           "subset_5000_device_poses_per_s": len(few) / dt_dev_few,
           "subset_5000_plain_100_pose_items_poses_per_s": len(few) / dt_items,
           "speedup_vs_plain_100_pose_items": dt_items / dt_dev_few,
           "items_equal_device": bool(np.array_equal(r4, r5, equal_nan=True)),
           "device_equals_plain": bool(np.array_equal(r1, r2, equal_nan=True)),
           "evals_per_pose_mean": float(n1.mean()),
           "start_E_median": float(np.median(e0)), "minimized_E_median": float(np.median(r1[:, 0])),
           "lowered_fraction": float(np.mean(r1[:, 0] < e0)),
           # poses whose last evaluation is the start pose again: deep clashes whose
           # gradient is so large that VA13's line search shrinks the step below the
           # FP32 resolution of the DOFs (the reference minimizer stalls the same way)
           "ended_at_start_energy_fraction": float(np.mean(r1[:, 0] == e0)),
           "final_nan_fraction": float(np.mean(~np.isfinite(r1[:, 0]))),
           "start_no_contact_fraction": float(np.mean(e0 == 0)),
           "reference_order": reference_order}
    if with_cpu:
        # the reference's order with the host's sin/cos against the oracle as
        # the reference runs it (libm sin/cos), 64 poses
        from oracle import pyoracle as po
        few = np.ascontiguousarray(sub[:64])
        ctx.set_kernel_options(kopts | KOPT_REFERENCE_ORDER)
        ctx.set_host_sincos(4096.0)
        ctx.minimize_6d_modes(*ids, few[:8], max_evals=10)
        t0 = time.perf_counter()
        dev = ctx.minimize_6d_modes(*ids, few, max_evals=steps)
        dt = time.perf_counter() - t0
        ctx.set_host_sincos(0)
        ctx.set_kernel_options(kopts)
        hr, hl = ctx.download_grid(gr), ctx.download_grid(gl)
        ref = po.minimize_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, few, steps)
        reference_order.update({
            "minimize_sample_poses": len(few), "minimize_poses_per_s": len(few) / dt,
            "minimize_bitwise_equal_oracle": bool(all(np.array_equal(a, b, equal_nan=True)
                                                      for a, b in zip(dev, ref))),
            "minimize_agreement_within_1e-3": po.minimization_stats(dev[1], ref[1])["within_tol"],
            "minimize_default_order_agreement_within_1e-3": po.minimization_stats(r1[:64], ref[1])["within_tol"]})
    for i in (gr, gl, lig, rec, par):
        ctx.release(i)
    return res


def bench_adjoint(ctx, pkg, n_poses: int):
    """Config 3: pairwise energy forward + hand-written adjoint (autograd) evals/s."""
    import torch
    from gbattract.autograd import PairwiseEnergy, PairwiseSystem
    wl = pkg.synth.make_config(3, n_poses=n_poses)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    grid = ctx.build_grid(rec, par, pkg.GridOptions())
    rng = np.random.default_rng(3)
    T = 32
    sysm = PairwiseSystem(ctx=ctx, rec=rec, lig=lig, grid=grid,
                          ipon=torch.ones((T, T), dtype=torch.int32, device="cuda"),
                          ffelec=wl.params.ffelec)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().requires_grad_(True)
    d, ql, qr = t(wl.dofs), t(wl.lig.charge), t(wl.rec.charge)
    r0, eps = t(rng.uniform(3, 5, (T, T))), t(rng.uniform(0.1, 10, (T, T)))

    def fb():
        for x in (d, ql, qr, r0, eps):
            x.grad = None
        E = PairwiseEnergy.apply(d, ql, qr, r0, eps, sysm)
        E.sum().backward()

    def fwd():
        with torch.no_grad():
            PairwiseEnergy.apply(d, ql, qr, r0, eps, sysm)

    rates, secs = {}, {}
    for name, f in (("fwd_bwd_evals_per_s", fb), ("fwd_evals_per_s", fwd)):
        f()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        secs[name] = (time.perf_counter() - t0) / 3
        rates[name] = len(wl.dofs) / secs[name]
    # algorithmic bytes: the pairwise kernels walk the same neighbour lists as
    # the grid kernel's census counts them; per pose 24 B DOF + 8 B per NL voxel
    # + 28 B per list entry (index, receptor xyz and charge, type, pairwise
    # charge), + 4 B energy (forward) or 4 B upstream gradient + 24 B dE/dDOF
    # (backward); per-bead and per-type-pair constants count once per call
    cen, _ = ctx.census_6d(rec, lig, grid, par, d.detach())
    cen = cen.cpu().numpy().astype(np.float64)
    walk = 8 * cen[:, 2].mean() + 28 * cen[:, 3].mean()
    peak, kind = measured_peaks()
    n = len(wl.dofs)
    t_f = secs["fwd_evals_per_s"]
    t_b = max(secs["fwd_bwd_evals_per_s"] - t_f, 1e-9)
    roof = {"forward": {"achieved": (28 + walk) * n / t_f / 1e9}, "backward": {"achieved": (52 + walk) * n / t_b / 1e9}}
    for v in roof.values():
        v.update({"peak": peak, "unit": "GB/s", "frac": v["achieved"] / peak, "peak_source": kind})
    roof["bytes_per_eval_walk"] = walk
    roof["note"] = ("wall time of synchronised calls; backward = forward+backward minus forward; "
                    "the pair arithmetic (LJ, Coulomb and their parameter derivatives) bounds these "
                    "kernels before memory does")
    for i in (grid, lig, rec, par):
        ctx.release(i)
    return {"workload": f"config 3: receptor {wl.rec.n} / ligand {wl.lig.n} beads, {len(wl.dofs)} poses, "
                        "10 A pairwise cutoff", **rates, "roofline": roof,
            "timing": "wall clock of 3 synchronised torch.autograd calls"}


def bench_batched_uneven(ctx, pkg, pose_scale: float, steps: int, plain_every: int = 1, tune: bool = True,
                         with_cpu: bool = True, nthreads: int = 1):
    """Config 4: 64 pairs of uneven sizes, each with its own grids, minimized in
    one persistent launch (default launch shapes, then the shapes gba_autotune
    picks per pair) against the plain per-step form run pair after pair on
    every plain_every-th pair (the same pairs timed batched), with per-pair
    completion times and, on a seeded sample, the symmetric agreement of the
    minimized energies with the CPU oracle's VA13."""
    import torch
    t_start = time.perf_counter()
    pairs = pkg.synth.make_batch(n_pairs=64, pose_scale=pose_scale)
    jobs, handles = [], []
    for wl in pairs:
        rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
        grid = ctx.build_grid(rec, par, pkg.GridOptions())
        handles += [grid, lig, rec, par]
        jobs.append((rec, lig, grid, par, wl.dofs))
    torch.cuda.synchronize()
    total = sum(len(j[4]) for j in jobs)
    # octet copies (cooperative lookups) for the pairs with the most poses while
    # more than 80 GB of device memory stays free: all 64 would need ~320 GB
    octet_pairs = 0
    for k in sorted(range(len(jobs)), key=lambda k: -len(jobs[k][4])):
        if torch.cuda.mem_get_info()[0] < 80e9:
            break
        ctx.grid_octets(jobs[k][2], True)
        octet_pairs += 1
    setup_s = time.perf_counter() - t_start
    log(f"config 4: {total} poses, grids and octets {setup_s:.1f} s")
    ctx.batch_minimize_6d([(*j[:4], j[4][:8]) for j in jobs], max_evals=5)      # warm-up

    def timed(js):
        t0 = time.perf_counter()
        got = ctx.batch_minimize_6d(js, max_evals=steps, done_ns=True)
        dt = time.perf_counter() - t0
        return got, dt, np.array([g[3].max() / 1e6 for g in got])

    got_u, dt_u, ms_u = timed(jobs)
    log(f"config 4: batched, default shapes {dt_u:.1f} s")
    res = {"workload": f"config 4: 64 pairs, receptor 300-3000 / ligand 100-1500 beads, {total} poses "
                       f"(pose counts x{pose_scale}), maxFunEval {steps}; octet grids for {octet_pairs} pairs",
           "batched_default_shapes_poses_per_s": total / dt_u,
           "batched_default_shapes_pair_completion_ms_p50": float(np.percentile(ms_u, 50)),
           "batched_default_shapes_pair_completion_ms_p99": float(np.percentile(ms_u, 99))}
    got, ms = got_u, ms_u
    if tune:
        cache = str(Path("/tmp") / "gba_tune_cache.txt")
        t0 = time.perf_counter()
        shapes = [ctx.autotune(*j[:4], j[4][:512], max_evals=20, cache_path=cache) for j in jobs]
        tune_s = time.perf_counter() - t0
        got, dt_t, ms = timed(jobs)
        log(f"config 4: autotune {tune_s:.1f} s, batched with tuned shapes {dt_t:.1f} s")
        kinds = {}
        for sh in shapes:
            k = f"{sh['minimize_threads']}x{sh['minimize_chunk']}"
            kinds[k] = kinds.get(k, 0) + 1
        res.update({"autotune_s": tune_s, "tuned_minimize_shapes": kinds,
                    "tuned_energy_threads": sorted({sh["energy_threads"] for sh in shapes}),
                    "batched_tuned_poses_per_s": total / dt_t,
                    "tuned_gain": dt_u / dt_t,
                    "tuned_equals_default": bool(all(np.array_equal(a[1], b[1]) for a, b in zip(got, got_u)))})
    res["batched_device_poses_per_s"] = total / (dt_t if tune else dt_u)
    res["batched_pair_completion_ms_p50"] = float(np.percentile(ms, 50))
    res["batched_pair_completion_ms_p99"] = float(np.percentile(ms, 99))
    # the plain per-step form (one launch per evaluation round, host VA13),
    # pair after pair, against the batched form on the same pairs
    sub = jobs[::plain_every]
    n_sub = sum(len(j[4]) for j in sub)
    got_sub, dt_dev_sub, _ = timed(sub) if plain_every > 1 else (got, total / res["batched_device_poses_per_s"], None)
    t0 = time.perf_counter()
    plain_done, plain = [], []
    for (rec, lig, grid, par, dofs) in sub:
        plain.append(ctx.minimize_6d_plain(rec, lig, grid, par, dofs, max_evals=steps))
        plain_done.append(1e3 * (time.perf_counter() - t0))
    dt_plain = time.perf_counter() - t0
    log(f"config 4: plain per-step form on {len(sub)} pairs {dt_plain:.1f} s")
    pd = np.array(plain_done)
    res.update({"plain_pairs": len(sub), "plain_poses": n_sub,
                "plain_per_step_poses_per_s": n_sub / dt_plain,
                "batched_same_pairs_poses_per_s": n_sub / dt_dev_sub,
                "speedup": dt_plain / dt_dev_sub,
                "device_equals_plain": bool(all(np.array_equal(a[1], b[1]) for a, b in zip(got_sub, plain))),
                "plain_pair_completion_ms_p50": float(np.percentile(pd, 50)),
                "plain_pair_completion_ms_p99": float(np.percentile(pd, 99))})
    # the reference's own execution model: 100-pose work items, one launch
    # each, per evaluation round (src/server/Server.h:39), on two pairs
    few = [jobs[k] for k in (len(jobs) // 3, 2 * len(jobs) // 3)]
    n_few = sum(len(j[4]) for j in few)
    got_few, dt_dev_few, _ = timed(few)
    t0 = time.perf_counter()
    items = [ctx.minimize_6d_plain(*j[:4], j[4], max_evals=steps, item_size=100) for j in few]
    dt_items = time.perf_counter() - t0
    log(f"config 4: 100-pose work items on 2 pairs {dt_items:.1f} s")
    res.update({"items_pairs": len(few), "items_poses": n_few,
                "plain_100_pose_items_poses_per_s": n_few / dt_items,
                "batched_items_pairs_poses_per_s": n_few / dt_dev_few,
                "speedup_vs_plain_100_pose_items": dt_items / dt_dev_few,
                "items_equal_device": bool(all(np.array_equal(a[1], b[1]) for a, b in zip(got_few, items)))})
    if with_cpu:
        # agreement with the CPU oracle's VA13: 32 seeded poses of every 8th pair
        from oracle import pyoracle as po
        rng = np.random.default_rng(404)
        dev, ref = [], []
        for k in range(0, len(jobs), 8):
            rec, lig, grid, par, dofs = jobs[k]
            idx = np.sort(rng.choice(len(dofs), 32, replace=False))
            gh = ctx.download_grid(grid)
            _, r_cpu, _ = po.minimize_6d(pairs[k].rec, pairs[k].lig, gh, pairs[k].params, dofs[idx], steps,
                                         nthreads=nthreads)
            dev.append(got[k][1][idx])
            ref.append(r_cpu)
        res["oracle_sample"] = {"poses": int(sum(len(r) for r in ref)), "pairs": len(ref),
                                **po.minimization_stats(np.concatenate(dev), np.concatenate(ref))}
    for i in handles:
        ctx.release(i)
    res["section_s"] = time.perf_counter() - t_start
    return res


def run_modes_only(args):
    """`--suite modes`: the config-2 section alone (profiling captures of the
    modes kernel); --no-min skips the minimizers."""
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    pkg = __graft_entry__.load_package()
    from gbattract.context import GbaContext
    ctx = GbaContext(0)
    ctx.set_kernel_options(args.kopts)
    res = bench_modes(ctx, pkg, n_poses=args.modes_poses, steps=200, minimize=not args.no_min,
                      with_cpu=not args.no_cpu, small=args.modes_small, kopts=args.kopts)
    ctx.close()
    print(json.dumps({"suite": {"modes": res}}))
    return 0


def run_section_only(args):
    """`--suite adjoint` / `--suite minimize` / `--suite batched`: the config-3,
    config-0 or config-4 section alone (profiling captures, section timings)."""
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    pkg = __graft_entry__.load_package()
    from gbattract.context import GbaContext
    ctx = GbaContext(0)
    if args.suite == "adjoint":
        res = bench_adjoint(ctx, pkg, n_poses=args.poses or 10_000)
    elif args.suite == "batched":
        res = bench_batched_uneven(ctx, pkg, pose_scale=args.batch_scale, steps=500, plain_every=args.plain_every,
                                   with_cpu=not args.no_cpu, nthreads=os.cpu_count() or 1)
    else:
        res = bench_minimization(ctx, pkg, nthreads=os.cpu_count() or 1, with_cpu=not args.no_cpu)
    ctx.close()
    print(json.dumps({"suite": {args.suite: res}}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbattract", choices=["gbattract", "reference"])
    ap.add_argument("--poses", type=int, default=None, help="override the pose count")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-sample", type=int, default=2000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-min", action="store_true", help="skip the minimization reports (configs 0 and 4)")
    ap.add_argument("--no-batch", action="store_true", help="skip the config-4 report")
    ap.add_argument("--no-suite", action="store_true", help="skip the config-2 and config-3 reports")
    ap.add_argument("--suite", default="default",
                    choices=["default", "full", "modes", "adjoint", "minimize", "batched"],
                    help="default (= full): config 1 (timed), config 0 and config 4 minimization, "
                         "config 2 (modes) and config 3 (adjoint); modes / adjoint / minimize / batched: "
                         "config 2, 3, 0 or 4 alone")
    ap.add_argument("--modes-poses", type=int, default=50000)
    ap.add_argument("--modes-small", action="store_true",
                    help="config 2's distributions with a 700 / 300-bead pair (profiling captures)")
    ap.add_argument("--variant", default="order=1,octets=1",
                    help="layout / visiting-order variant timed, or 'search' to time all four "
                         "and keep the fastest")
    ap.add_argument("--rec-beads", type=int, default=None,
                    help="smaller receptor with config 1's distributions (profiling captures)")
    ap.add_argument("--kopts", type=int, default=15,
                    help="kernel options (GBA_KOPT_*: 1 computed ratio, 2 cooperative lookup, "
                         "4 four blocks per SM, 8 typed neighbour list)")
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="fraction of config 4's pose counts (1.0: the configuration as stated)")
    ap.add_argument("--plain-every", type=int, default=8,
                    help="config 4: the plain per-step form runs on every k-th pair (and the batched "
                         "form again on the same pairs for the speedup)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.suite == "modes":
        return run_modes_only(args)
    if args.suite in ("adjoint", "minimize", "batched"):
        return run_section_only(args)

    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import __graft_entry__
    pkg, wl = make_workload(args.poses * world if args.poses else (100_000 * world if world > 1 else None),
                            args.rec_beads)
    wl.dofs = np.ascontiguousarray(shard(wl.dofs, world, rank))
    from gbattract.context import GbaContext
    ctx = GbaContext(local)
    ctx.set_kernel_options(args.kopts)
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
                       24 * cen[:, 3].sum())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        ctx.energy_6d(rec, lig, grid, par, dofs, out=out, stream=sptr)

    def timed_ms(reps=3):
        ts = []
        for _ in range(reps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return min(ts)

    # layout / visiting-order variants (short runs); the fastest is timed below
    variants = {}
    ref_out = None
    combos = [(o, c) for o in (False, True) for c in (False, True)]
    if args.variant != "search":
        kv = dict(x.split("=") for x in args.variant.split(","))
        combos = [(kv.get("order", "1") == "1", kv.get("octets", "1") == "1")]
    for order, octets in combos:
        ctx.set_pose_order(order)
        ctx.grid_octets(grid, octets)
        step()
        torch.cuda.synchronize()
        if ref_out is None:
            ref_out = out.clone()
        elif not torch.equal(out, ref_out):
            raise RuntimeError("variant changed the results")
        variants[f"order={int(order)},octets={int(octets)}"] = timed_ms()
    best = min(variants, key=variants.get)
    ctx.set_pose_order(best.startswith("order=1"))
    ctx.grid_octets(grid, best.endswith("octets=1"))
    log("variants (ms): " + json.dumps(variants) + " -> " + best)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    times = []
    # CUDA events around the energy kernel itself, recorded by the library on
    # the launching stream (the step also runs the visiting-order pass)
    ctx.kernel_timing(True)
    ctx.kernel_time(reset=True)
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
    kernel_ms, kernel_launches = ctx.kernel_time(reset=True)
    ctx.kernel_timing(False)
    ks = [a.elapsed_time(b) / 1000.0 for a, b in times]
    ktot, = max_over_ranks([sum(ks)], world)
    value = world * n * args.steps / ktot
    kavg = ktot / args.steps
    kernel_avg_s = kernel_ms / 1000.0 / max(1, kernel_launches)
    achieved = bytes_launch / kernel_avg_s / 1e9
    tpp, traffic_src = traffic_per_pose(f"{best},kopts={args.kopts}")
    traffic = None if tpp is None else tpp * n
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
    e2e_dt, = max_over_ranks([(time.perf_counter() - t0) / e_steps], world)
    e2e = world * n / e2e_dt

    # parity spot check of the timed result (device path) against the host path
    ok = bool(np.array_equal(out.cpu().numpy(), ho.numpy()))

    # the same batch summed in the reference CPU path's order (outside the
    # timed region; the timed result is kept in `out` for the parity check)
    reference_order = None
    ro_result = None
    if not args.kopts & KOPT_REFERENCE_ORDER:
        keep = out.clone()
        ctx.set_kernel_options(args.kopts | KOPT_REFERENCE_ORDER)
        step()
        torch.cuda.synchronize()
        ro_ms = timed_ms(2)
        ctx.set_kernel_options(args.kopts)
        reference_order = {"evals_per_s": n / (ro_ms / 1000.0), "ms_per_step": ro_ms,
                           "time_ratio": ro_ms / (1000.0 * kavg)}
        ro_result = out.cpu().numpy()
        out.copy_(keep)

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
        gh = ctx.download_grid(grid)
        nthreads = os.cpu_count() or 1
        rate, ns, dt = cpu_rate(pkg, wl, gh, args.cpu_seconds, nthreads)
        cpu = {"value": rate, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"first {ns} poses of the workload ({dt:.1f} s on {nthreads} threads)"}
        parity = timed_result_parity(wl, gh, out.cpu().numpy(), min(ns, 20000), nthreads, ro_result)

    l2_peak = measured_l2_peak() if rank == 0 else None
    minim = None
    if rank == 0 and not args.no_min:
        minim = bench_minimization(ctx, pkg, os.cpu_count() or 1, with_cpu=not args.no_cpu, kopts=args.kopts)
    batched = None
    if rank == 0 and not args.no_min and not args.no_batch:
        ctx.grid_octets(grid, False)
        batched = bench_batched_uneven(ctx, pkg, pose_scale=args.batch_scale, steps=500,
                                       plain_every=args.plain_every, with_cpu=not args.no_cpu,
                                       nthreads=os.cpu_count() or 1)
    suite = {}
    if rank == 0 and not args.no_suite:
        ctx.grid_octets(grid, False)
        suite["modes"] = bench_modes(ctx, pkg, n_poses=args.modes_poses, steps=200, with_cpu=not args.no_cpu,
                                     kopts=args.kopts)
        suite["adjoint"] = bench_adjoint(ctx, pkg, n_poses=10000)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * kavg, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD if not args.rec_beads else
                       f"config 1 distributions, receptor {wl.rec.n} / ligand {wl.lig.n} beads, {n} poses",
                       "poses": n, "receptor_beads": wl.rec.n,
                       "ligand_beads": wl.lig.n, "l2": "flushed (256 MB write) between steps",
                       "grid_MB": None},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(24 * n),
                    "d2h_bytes_per_step": int(28 * n)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                         "peak_source": peak_kind,
                         "bytes_per_launch": bytes_launch, "kernel_ms_avg": 1000.0 * kernel_avg_s,
                         "kernel_launches_timed": kernel_launches,
                         # the unique DRAM bytes of one launch (ncu) over the same kernel time
                         "dram": None if traffic is None else {
                             "achieved": traffic / kernel_avg_s / 1e9, "peak": peak,
                             "frac": traffic / kernel_avg_s / 1e9 / peak},
                         "l2": None if l2_peak is None else {
                             "achieved": achieved, "peak": l2_peak, "frac": achieved / l2_peak,
                             "peak_source": "measured in this run: graph of 50 copies of a 2 x 48 MB L2-resident "
                                            "working set"}},
            "parity": parity,
            "cpu_baseline": cpu, "clocks": clk.summary(),
            # per step: the fused energy kernel (+ the three visiting-order kernels --
            # cell counts, their prefix sum, the scatter -- when the order is on)
            "gpu_launches": args.steps * (4 if best.startswith("order=1") else 1),
            "reference_order": reference_order,
            "minimization": minim,
            "batched_uneven": batched,
            "variants_ms": variants, "variant_timed": best, "kernel_options": args.kopts,
            "suite": suite or None,
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
