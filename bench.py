"""Benchmark: particle-steps/s of the DEM contact step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the polydisperse settle -- 1,000,000 spheres, r ~ U[2, 4] mm,
rejection-sampled without overlap in a 1 x 1 x 2 m box of five plane walls,
dt = 5e-6 s, the reference's grid (origin -1, 128^3 cells of 2 x r_max), seeded
synthetic input.  A step is one whole DEM step (VV position, hash, sort, cell
ranges, particle-particle, planes, VV velocity).

Our arm (default) prints one JSON line with:
  value      particle-steps/s with the state resident in HBM (device timed,
             CUDA events on the launching stream; the state, ~190 MB, is
             larger than L2, so no flush is needed between steps);
  e2e        the same metric through the C ABI with host buffers: every step
             uploads the evolving state from pinned host memory, steps once
             and downloads pos/vel/omega/acc/alpha;
  roofline   the particle-particle kernel's algorithmic bytes (140 B/particle)
             over its live event-timed duration vs the measured HBM peak;
  cpu_baseline  the reference's CPU path (restated in the oracle, single
             thread) on a bounded sample of the same scene.
--impl reference runs that CPU path on the host cores instead (one scene
replica per core) and prints the same metric.
Under torchrun each rank advances its own replica (scenes shard with no
exchange); value is the sum over ranks over the max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
WORKLOAD = "polydisperse_box_settle"
B_CONTACT = {"fp64": 140, "mixed": 116}   # algorithmic bytes per particle, contact kernel
# k_mx_advance (the mixed form's dominant kernel), per particle and middle step:
# reads x y z r (32), vh vl wh wl ab (80), b2 (8), Fc Mc (32), pref (16) = 168;
# writes x y z (24), vh vl wh wl ab (80), b2 (8), pf qa qb (48) = 160.
B_ADVANCE = 328


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000, help="spheres (default: the 1M scene)")
    ap.add_argument("--cpu-steps", type=int, default=0, help="CPU-baseline sample steps (0: auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"],
                    help="scene form for the headline value (the other is reported beside it)")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 side measurement")
    return ap.parse_args()


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_from_profiles(name):
    """Per-launch DRAM bytes of a kernel from its committed ncu summary."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("traffic_bytes_per_launch_full_scene:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def _scene(n):
    """The benchmark scene (cached in the temp directory: generation is ~15 s)."""
    import tempfile

    import numpy as np

    from metakonga_gb300 import scenes
    path = os.path.join(tempfile.gettempdir(), f"xdem_polydisperse_box_{n}_seed7.npz")
    if os.path.exists(path):
        try:
            z = np.load(path)
            sc = scenes.polydisperse_box(n=min(n, 64))      # template for walls/params
            sc.pos, sc.mass, sc.inertia = z["pos"], z["mass"], z["inertia"]
            for k in ("vel", "acc", "omega", "alpha", "moment"):
                setattr(sc, k, np.zeros((n, 3)))
            sc.force = z["force"]
            sc.planes = z["planes"].view(sc.planes.dtype)
            sc.params = z["params"].view(sc.params.dtype).reshape(())
            return sc
        except Exception:
            pass
    sc = scenes.polydisperse_box(n=n)
    try:
        np.savez(path, pos=sc.pos, mass=sc.mass, inertia=sc.inertia, force=sc.force,
                 planes=sc.planes.view(np.uint8), params=sc.params.reshape(1).view(np.uint8))
    except OSError:
        pass
    return sc


def _cpu_worker(args):
    """One CPU-path replica (spawned process): builds the scene once, then
    times `samples` runs of `steps` steps; returns (particles*steps, [seconds])."""
    n, steps, samples = args
    sys.path.insert(0, ROOT)
    from oracle.pyoracle import Oracle
    sc = _scene(n)
    o = Oracle()
    times = []
    for _ in range(samples):
        t0 = time.perf_counter()
        o.run(sc, steps, cpu_path=True)
        times.append(time.perf_counter() - t0)
    return n * steps, times


def cpu_baseline(n, steps, procs=1, samples=1):
    """Reference CPU path throughput: procs replicas, each timing `samples`
    runs of `steps` steps; per sample, value = procs * n * steps / slowest."""
    import multiprocessing as mp
    if procs == 1:
        done, times = _cpu_worker((n, steps, samples))
        return [done / t for t in times], times
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_worker, [(n, steps, samples)] * procs)
    vals, walls = [], []
    for i in range(samples):
        wall = max(r[1][i] for r in res)
        vals.append(sum(r[0] for r in res) / wall)
        walls.append(wall)
    return vals, walls


def run_reference(a):
    world, rank, _ = _dist()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    steps = a.cpu_steps or 1
    t0 = time.perf_counter()
    vals, walls = cpu_baseline(a.n, steps, procs=cores, samples=a.warmup + a.steps)
    vals = vals[a.warmup:]
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * a.n / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded MT19937 rejection-sampled spheres)",
        "config": {"workload": WORKLOAD, "particles": a.n, "dt": 5e-6, "grid": "128^3 wrapped",
                   "l2": "state > L2 (no flush)"},
        "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{steps} step(s) of the {a.n}-sphere scene per sample, one "
                                   f"single-threaded replica per core ({cores})"},
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line), flush=True)


def _time_scene(sc, mode, steps, warmup, stream, barrier, world, with_clock, local):
    """Device-timed steps of one scene form; returns (ms, phases, launches, clocks,
    scene, cell re-binnings in the timed steps).

    The timed run has phase timing off (so the mixed form replays its CUDA
    graphs); a second run of the same length records per-phase CUDA events."""
    import torch

    from metakonga_gb300 import engine
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED if mode == "mixed" else engine.MODE_FP64)
    sh = stream.cuda_stream
    ds.step(warmup, check=True, stream=sh)
    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local) if with_clock else None
    if clk:
        clk.__enter__()
    rb0, rb_each = ds.rebuilds(sh)
    barrier()
    ev0.record(stream)
    ds.step(steps, check=False, stream=sh)
    ev1.record(stream)
    barrier()
    if clk:
        clk.__exit__(None, None, None)
    ms = ev0.elapsed_time(ev1)
    rebuilds = ds.rebuilds(sh)[0] - rb0
    launches = ds.launches(steps) + rebuilds * rb_each
    ds.set_timing(True)
    ds.step(steps, check=False, stream=sh)
    phases = ds.phase_times()
    ds.set_timing(False)
    # a one-step call: its phase totals, taken from a K-step call's, leave
    # K - 1 steps' worth without the once-per-call final velocity update
    ds.set_timing(True)
    ds.step(1, check=False, stream=sh)
    one = ds.phase_times()
    ds.set_timing(False)
    phases["_one"] = one
    barrier()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, phases, launches, (clk.summary() if clk else None), ds, rebuilds


def run_ours(a):
    import numpy as np
    import torch

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sc = _scene(a.n)
    n = a.n
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    with torch.cuda.stream(stream):
        ms, phases, launches, clocks, ds, rebuilds = _time_scene(sc, a.mode, a.steps, a.warmup, stream,
                                                                 barrier, world, True, local)
    value = world * n * a.steps / (ms / 1e3)

    # e2e: through the C ABI with pinned host buffers, state round trip every step
    host = {k: torch.from_numpy(np.ascontiguousarray(getattr(sc, k))).pin_memory() for k in
            ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")}
    outs = {k: torch.empty_like(host[k]).pin_memory() for k in ("pos", "vel", "acc", "omega", "alpha")}
    from metakonga_gb300._lib import call
    up_keys = ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")
    up = [host[k].data_ptr() for k in up_keys]
    h2d = sum(host[k].numel() * 8 for k in up_keys)
    d2h = sum(outs[k].numel() * 8 for k in outs)
    e2e_steps = max(3, min(a.steps, 10))

    def e2e_step():
        call("xd_scene_upload", ds.handle, *up, sh)
        call("xd_scene_step", ds.handle, 1, 0, sh)
        call("xd_scene_download", ds.handle, outs["pos"].data_ptr(), outs["vel"].data_ptr(),
             outs["acc"].data_ptr(), outs["omega"].data_ptr(), outs["alpha"].data_ptr(), None,
             None, sh)

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * n * e2e_steps / e2e_s
    ds.close()

    one = phases.pop("_one")
    peak, peak_kind = _peaks()
    c_ms, c_n = phases["p2p"]
    contact = {"avg_launch_ms": c_ms / c_n if c_n else None}
    if a.mode == "mixed":
        # dominant kernel: the in-place advance (velocity-Verlet, contact view, skin test)
        k_ms = (phases["vv"][0] - one["vv"][0]) / max(a.steps - 1, 1)
        bpp = B_ADVANCE
        kname = "k_mx_advance<1> (in-place velocity-Verlet, contact view, skin test)"
        traffic = _traffic_from_profiles("advance_mixed_polydisperse_box.md")
        contact.update({"kernel": "k_mx_contact (Verlet-list pairs and planes of the heavy list)",
                        "traffic": _traffic_from_profiles("contact_mixed_polydisperse_box.md"),
                        "bytes_per_particle_full_pass": B_CONTACT["mixed"],
                        "achieved_full_pass_gbs": (n * B_CONTACT["mixed"]) / (c_ms / c_n / 1e3) / 1e9
                        if c_n else None})
    else:
        k_ms = c_ms / c_n if c_n else None
        bpp = B_CONTACT["fp64"]
        kname = "k_p2p (FP64 particle-particle)"
        traffic = _traffic_from_profiles("p2p_fp64_polydisperse_box.md")
    achieved = (n * bpp) / (k_ms / 1e3) / 1e9 if k_ms else None
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
            "traffic": traffic, "bytes_per_particle": bpp, "avg_launch_ms": k_ms,
            "contact_pass": contact}
    phase_ms = {k: round(v[0] / max(v[1], 1), 4) for k, v in phases.items() if v[1]}

    plain = None
    if not a.no_plain:
        other = "fp64" if a.mode == "mixed" else "mixed"
        psteps = max(3, min(a.steps, 10))
        with torch.cuda.stream(stream):
            pms, pph, _, _, pds, _ = _time_scene(sc, other, psteps, 1, stream, barrier, world, False,
                                                 local)
        pds.close()
        pph.pop("_one", None)
        plain = {"mode": other, "value": world * n * psteps / (pms / 1e3), "steps": psteps,
                 "ms_per_step": pms / psteps,
                 "phase_ms_per_launch": {k: round(v[0] / max(v[1], 1), 4) for k, v in pph.items() if v[1]}}

    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        csteps = a.cpu_steps or 3
        vals, times = cpu_baseline(n, csteps, procs=1, samples=1)
        cpu = {"value": vals[0], "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"{csteps} steps of the same {n}-sphere scene, reference CPU path "
                         f"(restated, single thread), {times[0]:.1f} s"}
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if a.mode == "fp64" else "f64+f32",
        "data": "synthetic (seeded MT19937 rejection-sampled spheres)",
        "config": {"workload": WORKLOAD, "particles": n, "dt": 5e-6, "mode": a.mode,
                   "grid": ("128^3 wrapped, cell 8 mm" if a.mode == "fp64" else
                            "scene grid sized to the box, cell 2 r_max"),
                   "l2": "state > L2 (no flush)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "cell_rebinnings_in_timed_steps": rebuilds,
        "roofline": roof,
        "phase_ms_per_launch": phase_ms,
        "other_form": plain,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
