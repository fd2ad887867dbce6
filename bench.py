"""Benchmark: particle-steps/s of the DEM contact step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batched|served|box|drum|hopper]

Workloads (seeded synthetic input; every scene is generated here):
  batched  (default) 256 independent hopper-discharge scenes: particle counts
           log-uniform in [2,000, 200,000] (11.56 M spheres in all), r ~ U[2, 4]
           mm, a 60-degree cone of 4,096 triangles above a plane floor, orifice
           U[6, 12] diameters, friction U[0.2, 0.6], dt = 5e-6 s.  Each hopper
           is generated as a lattice with its orifice gated, settled into a bed
           (metakonga_gb300.prepare.settle, untimed), and the gate opened: the
           timed steps are the discharge of packed beds.  A step advances every
           scene by one time step through one batch (xd_batch) in the mixed
           form.
  served   a Poisson stream of settle-box and hopper requests, particle counts
           log-uniform in [1,000, 500,000], step counts U[1,000, 20,000],
           admitted under a 150 GB device-memory budget by the continuous-
           batching server; p50/p99 completion latency and particle-steps/s.
  box      the 1,000,000-sphere polydisperse settle (r ~ U[2, 4] mm in a
           1 x 1 x 2 m box of five plane walls, dt = 5e-6 s), one scene.
  drum     the 500,000-sphere rotating drum (20,480 triangles turning).
  hopper   one settled hopper (--hopper-n spheres, the batch's preparation,
           cached in the temp directory): the contact-pass profiles' workload.

The default (batched) line carries:
  value        particle-steps/s of the settled batch, device-timed (CUDA
               events on the launching stream; the batch's state, ~15 GB, is
               far larger than L2, so no flush is needed between steps);
  e2e          the same through the public API with host buffers: each
               scene's state uploaded from pinned host memory, K steps, the
               state downloaded (all inside the timed region);
  roofline     the batch step's dominant kernel -- the contact pass
               (k_batch_contact: the cooperative pair pass and the wall pass
               over every scene's listed spheres) on packed beds,
               k_batch_advance<1> otherwise -- timed per launch with CUDA
               events, its algorithmic bytes over that time against the
               measured HBM peak; both kernels' figures are under "kernels";
  autotune     the autotuner's choice on the particle-weighted median scene
               and the batch's time with it against the defaults;
  step_beyond_kernels_ms  a step's time outside its advance, pair and wall
               launches (re-binnings, decisions, graph nodes);
  lattice_start the same batch from its generated lattice (little contact),
               and after 4,000 steps of falling ("fallen_4000");
  plain_fp64   the same scenes run one at a time in the FP64 form (the
               reference's algorithm and grid), and the ratio to it;
  fp64_check   per-particle contact-force error of the mixed form against the
               FP64 form on the median scene's settled bed;
  single_scene_box, settle_8000, drum  those workloads' own figures (the
               box with the FP64 form on the reference's and on an unwrapped
               grid);
  served       the served stream stepped side by side (p50/p99 ms,
               particle-steps/s), the same stream in cohorts, a sweep of
               arrival rates with --rates, and the same requests' time alone
               in the FP64 form;
  cpu_baseline the reference's CPU path (restated in the oracle, one thread)
               on the median scene's settled bed.
--impl reference runs that CPU path on the host cores instead (one replica of
the median scene per core) and prints the same metric.
Under torchrun each rank advances its own replica of the workload (scenes
shard with no exchange); value is the sum over ranks over the max rank time.
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
# scenes of a batch overlap on 32 library streams: give them 32 hardware
# queues (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "particle-steps/s"
WORKLOAD = "polydisperse_box_settle"
BATCH_WORKLOAD = "hopper_batch_256"
SERVED_WORKLOAD = "served_settle_and_hopper_requests"
B_CONTACT = {"fp64": 140, "mixed": 116}   # algorithmic bytes per particle, contact kernel
# k_mx_advance (the mixed form's dominant kernel), per particle and middle step:
# reads x y z r (32), vh vl wh wl ab (80), b2 (8), Fc Mc (32), pref (16) = 168;
# writes x y z (24), vh vl wh wl ab (80), b2 (8), pf qa qb pr (64) = 176.
B_ADVANCE = 344
# k_batch_contact / k_mx_contact, per listed sphere: reads pf 16, qa qb 32, pr 16, vh vl 32, wh wl 32,
# hlist 4, vcount 4, tcount 4, wmask 2; writes Fc Mc 32 = 174 B; plus 4 B per list entry
B_LISTED = 174


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000, help="spheres (default: the 1M scene)")
    ap.add_argument("--cpu-steps", type=int, default=0, help="CPU-baseline sample steps (0: auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"],
                    help="scene form for the headline value (the other is reported beside it)")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 side measurement")
    ap.add_argument("--workload", default="batched", choices=["batched", "served", "box", "drum", "hopper"])
    ap.add_argument("--hopper-n", type=int, default=100_000, help="hopper workload: spheres")
    ap.add_argument("--no-served", action="store_true", help="batched: skip the served stream")
    ap.add_argument("--no-box", action="store_true", help="batched: skip the 1M-box roofline run")
    ap.add_argument("--no-drum", action="store_true", help="batched: skip the rotating-drum run")
    ap.add_argument("--prep-steps", type=int, default=5000,
                    help="settled beds: preparation steps (prepare.settle) before the timed run (0: none)")
    ap.add_argument("--prep-dt", type=float, default=4e-5, help="time step of the preparation")
    ap.add_argument("--prep-cache", action="store_true",
                    help="keep the settled batch in the temp directory and load it when present")
    ap.add_argument("--no-lattice", action="store_true", help="batched: skip the lattice-start timing")
    ap.add_argument("--count", type=int, default=256, help="scenes in the batch")
    ap.add_argument("--requests", type=int, default=32, help="requests of the served stream")
    ap.add_argument("--rate", type=float, default=4.0, help="served arrivals per second")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="served device-memory budget")
    ap.add_argument("--chunk", type=int, default=50, help="served steps per scene per tick")
    ap.add_argument("--rates", default="", help="served: comma-separated arrival rates to sweep")
    ap.add_argument("--no-tune", action="store_true", help="batched: default tuning, no autotuner run")
    ap.add_argument("--tune-steps", type=int, default=200, help="batched: autotuner window (steps per candidate)")
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


def _traffic_from_profiles(name, key="traffic_bytes_per_launch_full_scene"):
    """Per-launch DRAM bytes of a kernel (or another figure named by key) from
    its committed ncu summary."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith(key + ":"):
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


def _cpu_scene(spec):
    """("box", n) -> the n-sphere polydisperse box; ("settle",) -> the
    8,000-sphere settle; ("scene", Scene) -> that scene as it stands."""
    from metakonga_gb300 import scenes
    if spec[0] == "box":
        return _scene(spec[1])
    if spec[0] == "settle":
        return scenes.settle_box()
    return spec[1]


def host_cpu():
    """The host CPU model and the cores this process may use."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.TimeoutExpired):
        pass
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count() or 1
    return {"cpu_model": model, "cores_available": cores}


def _cpu_worker(args):
    """One CPU-path replica (spawned process): its scene once, the oracle's
    grid work arrays once (outside the timed calls), then `samples` timed runs
    of `steps` steps; returns (particles * steps, [seconds])."""
    spec, steps, samples = args
    sys.path.insert(0, ROOT)
    from oracle.pyoracle import Oracle
    sc = _cpu_scene(spec)
    o = Oracle()
    work = o.work_arrays(sc)
    times = []
    for _ in range(samples):
        t0 = time.perf_counter()
        o.run(sc, steps, cpu_path=True, work=work)
        times.append(time.perf_counter() - t0)
    return sc.np_ * steps, times


def cpu_baseline(specs, steps, samples=1):
    """Reference CPU path throughput: one replica per spec (one spawned process
    each when there are several), each timing `samples` runs of `steps` steps;
    per sample, value = sum of particle-steps / slowest replica."""
    import multiprocessing as mp
    if len(specs) == 1:
        done, times = _cpu_worker((specs[0], steps, samples))
        return [done / t for t in times], times
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(specs)) as pool:
        res = pool.map(_cpu_worker, [(sp, steps, samples) for sp in specs])
    vals, walls = [], []
    for i in range(samples):
        wall = max(r[1][i] for r in res)
        vals.append(sum(r[0] for r in res) / wall)
        walls.append(wall)
    return vals, walls


def _median_index(specs):
    import numpy as np
    return int(np.argsort([d["n"] for d in specs])[len(specs) // 2])


def _settled_hoppers(specs, a, stream):
    """The batch's hoppers as settled beds with the orifice open: each scene
    generated with its gate closed, settled by prepare.settle (a.prep_steps
    steps of a.prep_dt in one batch), the gates then opened.  With
    a.prep_cache the settled states are kept in the temp directory (a
    profiler's run of the same workload then loads them instead of
    launching the preparation)."""
    import tempfile

    import numpy as np

    from metakonga_gb300 import prepare, scenes
    scs = [scenes.hopper(gate=True, **d) for d in specs]
    keys = ("pos", "vel", "acc", "omega", "alpha")
    path = os.path.join(tempfile.gettempdir(),
                        f"xdem_hopper_batch_{len(specs)}_{a.prep_steps}_{a.prep_dt:g}.npz")
    loaded = False
    if a.prep_cache and a.prep_steps:
        try:
            z = np.load(path)
            for k in keys:
                flat = z[k]
                off = 0
                for sc in scs:
                    arr = getattr(sc, k)
                    arr[:] = flat[off:off + arr.shape[0]]
                    off += arr.shape[0]
            loaded = True
        except (OSError, KeyError, ValueError):
            loaded = False
    if a.prep_steps and not loaded:
        prepare.settle(scs, a.prep_steps, dt=a.prep_dt, stream=stream)
        if a.prep_cache:
            try:
                np.savez(path, **{k: np.concatenate([getattr(sc, k) for sc in scs]) for k in keys})
            except OSError:
                pass
    prepare.open_gates(scs)
    return scs


def run_reference(a):
    """The reference's CPU path (the oracle's restatement, single-threaded as
    the reference is) on the host cores: one replica of the workload's median
    scene per core, in the same state as the GPU arm's cpu_baseline."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    host = host_cpu()
    cores = host["cores_available"]
    steps = a.cpu_steps or 10
    t0 = time.perf_counter()
    if a.workload == "box":
        spec = ("box", a.n)
        workload, cfg = WORKLOAD, {"particles": a.n, "grid": "128^3 wrapped"}
        n_one = a.n
        what = f"the {a.n}-sphere box"
    else:
        import torch

        from metakonga_gb300 import prepare, scenes
        specs = scenes.hopper_batch(count=a.count)
        k = _median_index(specs)
        sc = scenes.hopper(gate=True, **specs[k])
        if a.prep_steps:
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            prepare.settle(sc, a.prep_steps, dt=a.prep_dt)
        prepare.open_gates(sc)
        spec = ("scene", sc)
        n_one = sc.np_
        workload = BATCH_WORKLOAD if a.workload == "batched" else SERVED_WORKLOAD
        cfg = {"scenes": a.count, "grid": "128^3 wrapped, cell 2 x max(r, triangle circumradius)",
               "state": "settled bed, orifice open (prepare.settle on the GPU, untimed)"}
        what = (f"scene {k} of the {a.count}-scene batch ({n_one} spheres, the median; the GPU arm's "
                f"cpu_baseline scene)")
    vals, walls = cpu_baseline([spec] * cores, steps, samples=a.warmup + a.steps)
    vals = vals[a.warmup:]
    v = statistics.median(vals)
    sample = (f"{steps} steps per sample of {what}, one single-threaded replica per core ({cores}); "
              f"grid work arrays allocated once per replica, outside the timed calls")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * n_one * cores / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded MT19937 scenes)",
        "config": dict({"workload": workload, "dt": 5e-6, "l2": "state > L2 (no flush)"}, **cfg),
        "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample,
                         "per_core": v / cores, "host": host},
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


def _roofline(mode, n, steps, phases, one):
    """Roofline object of a scene's dominant kernel from its phase timings
    (phases: a K-step call's, one: a 1-step call's)."""
    peak, peak_kind = _peaks()
    c_ms, c_n = phases["p2p"]
    contact = {"avg_launch_ms": c_ms / c_n if c_n else None}
    if mode == "mixed":
        # dominant kernel: the in-place advance (velocity-Verlet, contact view, skin test)
        k_ms = (phases["vv"][0] - one["vv"][0]) / max(steps - 1, 1)
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
    return {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
            "traffic": traffic, "bytes_per_particle": bpp, "avg_launch_ms": k_ms,
            "contact_pass": contact}


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
    roof = _roofline(a.mode, n, a.steps, phases, one)
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
        vals, times = cpu_baseline([("box", n)], csteps, samples=1)
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
        "autotune": tuned,
        "step_beyond_kernels_ms": {"value": other_ms, "of_step": other_ms / (ms / a.steps),
                                   "note": "ms per batch step minus the advance and contact launches' live "
                                           "times: re-binnings, the decision kernel, run prefix, graph and "
                                           "conditional nodes -- the most a persistent kernel could save"},
        "roofline": roof,
        "phase_ms_per_launch": phase_ms,
        "other_form": plain,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def _torch_setup():
    import torch
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    return world, rank, local, barrier


def _max_over_ranks(x, world, device="cuda"):
    """The largest of the ranks' x (a time): the job ends with its slowest rank."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _fp64_alone(scs, steps, stream, own_grid=False):
    """Each scene alone in the plain FP64 form (one warm-up step, then `steps`
    device-timed steps): its ms per step.  own_grid: the particles on a grid
    of their own (cells of the largest diameter, unwrapped), the triangles on
    the reference's (xd_scene_set_particle_grid)."""
    import torch

    from metakonga_gb300 import engine
    sh = stream.cuda_stream
    out = []
    for sc in scs:
        d = engine.DeviceScene(sc, mode=engine.MODE_FP64)
        if own_grid:
            d.set_particle_grid()
        d.step(1, check=True, stream=sh)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        d.step(steps, check=False, stream=sh)
        e1.record(stream)
        e1.synchronize()
        out.append(e0.elapsed_time(e1) / steps)
        d.close()
    return out


def _fp64_check(sc, squeeze=0.92, seed=29, spin=True):
    """Contact forces of the mixed form against the FP64 form on one state:
    scene `sc` squeezed towards its centroid by `squeeze` (1: as it stands),
    with spin=True random velocities and spins; per particle
    |F_mixed - F_fp64| / max(|F_fp64|, m g) (stricter than the gate's
    max(sum_c |F_c|, m g): |F| <= sum_c |F_c|), and the same for the torque / r."""
    import numpy as np

    from metakonga_gb300 import engine
    st = sc.copy()
    if squeeze != 1.0:
        c = st.pos[:, :3].mean(axis=0)
        st.pos[:, :3] = c + (st.pos[:, :3] - c) * squeeze
    if spin:
        rng = np.random.Generator(np.random.MT19937(seed))
        st.vel[:] = rng.normal(0.0, 0.2, st.vel.shape)
        st.omega[:] = rng.normal(0.0, 20.0, st.omega.shape)
    out = []
    for mode in (engine.MODE_MIXED, engine.MODE_FP64):
        d = engine.DeviceScene(st, mode=mode)
        out.append(d.eval_contacts())
        d.close()
    (f_m, m_m), (f_r, m_r) = out
    den = np.maximum(np.linalg.norm(f_r, axis=1), st.mass * 9.81)
    err = np.linalg.norm(f_m - f_r, axis=1) / den
    r = st.pos[:, 3]
    merr = np.linalg.norm((m_m - m_r) / r[:, None], axis=1) / den
    touching = np.linalg.norm(f_r, axis=1) > 0
    state = (f"scene squeezed by {squeeze} towards its centroid" if squeeze != 1.0 else "the scene's state") + \
        (", velocities N(0, 0.2) m/s, spins N(0, 20) rad/s" if spin else "")
    return {"particles": int(st.np_), "touching": int(touching.sum()),
            "max_force_err": float(err.max()), "p999_force_err": float(np.percentile(err, 99.9)),
            "max_torque_over_r_err": float(merr.max()), "state": state,
            "normaliser": "max(|F_fp64|, m g) per particle",
            "gate_note": ("the parity tests gate at 2e-5 of max(sum_c |F_c|, m g); this normaliser is the net "
                          "force, about m g in a resting bed whose contacts each carry several m g, so it reads "
                          "a few times stricter there")}


def _box_roofline(a, stream, barrier, world, local):
    """The 1M-sphere box in the mixed form: value and the advance kernel's
    live roofline (its state streams from HBM every step)."""
    sc = _scene(1_000_000)
    import torch
    with torch.cuda.stream(stream):
        ms, phases, launches, _, ds, rebuilds = _time_scene(sc, "mixed", a.steps, a.warmup, stream,
                                                            barrier, world, False, local)
    ds.close()
    one = phases.pop("_one")
    roof = _roofline("mixed", sc.np_, a.steps, phases, one)
    roof["workload"] = ("polydisperse_box_settle, 1,000,000 spheres (one scene, launched directly for "
                        "its phase events: the batch's launches sit inside one graph per step, which "
                        "events cannot split)")
    out = {"value": world * sc.np_ * a.steps / (ms / 1e3), "ms_per_step": ms / a.steps,
           "gpu_launches": launches, "cell_rebinnings_in_timed_steps": rebuilds}
    if not a.no_plain:
        out["plain_fp64"] = _fp64_timed(sc, stream, 5)
        out["plain_fp64_own_grid"] = _fp64_timed(_own_grid(sc), stream, 5)
        out["plain_fp64_own_grid"]["grid"] = ("the FP64 form on a grid that holds the box unwrapped: cells of "
                                              "2 r_max, power-of-two dimensions covering the particles (the "
                                              "reference's 128^3 grid wraps the box's 250 cells of height onto "
                                              "128, two spheres' worth per cell)")
        out["ratio_to_plain_fp64_own_grid"] = out["value"] / out["plain_fp64_own_grid"]["value"]
    return roof, out


def _own_grid(sc):
    """The scene with a grid that covers its particles without wrapping:
    the reference's cell (2 r_max), power-of-two dimensions, the origin one
    cell below the lowest particle."""
    import numpy as np
    s = sc.copy()
    cell = float(sc.params["cell_size"])
    lo = sc.pos[:, :3].min(axis=0) - cell
    hi = sc.pos[:, :3].max(axis=0) + cell
    g = [1 << int(np.ceil(np.log2(max(2.0, (h - l) / cell)))) for l, h in zip(lo, hi)]
    s.params["grid"] = g
    s.params["ncell"] = int(np.prod(g))
    s.params["world_origin"] = lo
    return s


def _fp64_timed(sc, stream, steps, warmup=1):
    """The scene in the FP64 form: device time of `steps` steps after
    `warmup`."""
    import torch

    from metakonga_gb300 import engine
    d = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    d.step(warmup, check=True, stream=stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    d.step(steps, check=False, stream=stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    d.close()
    ms = e0.elapsed_time(e1) / steps
    return {"value": sc.np_ / (ms / 1e3), "ms_per_step": ms,
            "grid": [int(x) for x in sc.params["grid"]], "cell": float(sc.params["cell_size"])}


def _drum(a, stream, steps=200, warmup=3, plain=True):
    """The rotating drum at full size (500,000 spheres in a 20,480-triangle
    cylinder turning at 1 rad/s, the mesh moved on the device every step) in
    the mixed form, and the same scene's step time in the plain FP64 form."""
    import torch

    from metakonga_gb300 import engine, scenes
    sc = scenes.drum_lattice()
    sh = stream.cuda_stream
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.set_kinematic_bodies(True)
    ds.step(warmup, check=True, stream=sh)
    rb0 = ds.rebuilds(sh)[0]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ds.step(steps, check=False, stream=sh)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    rebuilds = ds.rebuilds(sh)[0] - rb0
    ds.close()
    value = sc.np_ * steps / (ms / 1e3)
    if not plain:
        return {"value": value, "unit": "particle-steps/s", "ms_per_step": ms / steps, "steps": steps,
                "cell_rebinnings_in_timed_steps": rebuilds}
    d64 = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    d64.set_kinematic_bodies(True)
    d64.step(1, check=True, stream=sh)
    e0.record(stream)
    d64.step(2, check=False, stream=sh)
    e1.record(stream)
    e1.synchronize()
    ms64 = e0.elapsed_time(e1) / 2
    d64.close()
    return {"workload": "rotating drum: 500,000 spheres r U[2,4] mm on a jittered FCC lattice from the "
                        "bottom, closed cylinder R 0.5 m L 0.4 m of 20,480 triangles turning at 1 rad/s "
                        "(kinematic on the device), wall friction 0.5, dt 5e-6",
            "value": value, "unit": "particle-steps/s", "ms_per_step": ms / steps, "steps": steps,
            "cell_rebinnings_in_timed_steps": rebuilds,
            "plain_fp64": {"value": sc.np_ / (ms64 / 1e3), "ms_per_step": ms64,
                           "method": "the same scene in the FP64 form (the reference's 128^3 grid of "
                                     "2 x max(r, triangle circumradius) cells, re-sorted every step), "
                                     "one warm-up step then 2 device-timed steps"},
            "ratio": value / (sc.np_ / (ms64 / 1e3))}


def _settle_small(stream, steps=1000, cpu=True):
    """The reference's CPU-runnable case: the 8,000-sphere lattice settle in a
    box of five planes (FP64, dt 1e-5) in both forms on the GPU, and the
    reference CPU path on the host beside it."""
    import torch

    from metakonga_gb300 import engine, scenes
    sc = scenes.settle_box()
    sh = stream.cuda_stream
    out = {"workload": "settle_box_8000: 20x20x20 lattice, pitch 11 mm, r 5 mm, five plane walls, dt 1e-5",
           "steps": steps}
    for name, mode in (("fp64", engine.MODE_FP64), ("mixed", engine.MODE_MIXED)):
        ds = engine.DeviceScene(sc, mode=mode)
        ds.step(3, check=True, stream=sh)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ds.step(steps, check=False, stream=sh)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        ds.close()
        out[name] = {"value": sc.np_ * steps / (ms / 1e3), "ms_per_step": ms / steps}
    if cpu:
        vals, times = cpu_baseline([("settle", 0)], 20)
        out["reference_cpu_path"] = {"value": vals[0], "cores": 1, "sample": f"20 steps, {times[0]:.2f} s"}
        out["fp64_vs_cpu"] = out["fp64"]["value"] / vals[0]
    return out


def _serve_once(scs, reqs, rate, a, stream, mode):
    """One served run of the request stream at `rate` arrivals per second;
    mode "cohorts" (batches per admission wave) or "side_by_side"."""
    from metakonga_gb300 import serve
    arrivals = serve.poisson_arrivals(len(reqs), rate, seed=5)
    srv = serve.Server(budget_bytes=int(a.budget_gb * 1e9), chunk=a.chunk, stream=stream.cuda_stream,
                       keep_results=True, cohorts=(mode == "cohorts"))
    for k, (r, sc) in enumerate(zip(reqs, scs)):
        srv.submit(k, sc, r["steps"], arrival=float(arrivals[k]))
    srv.run()
    rep = srv.report()
    return {"rate_per_s": rate, "mode": mode, "offered_particle_steps_per_s": rep["offered_particle_steps_per_s"],
            "particle_steps_per_s": rep["particle_steps_per_s"], "p50_ms": rep["p50_ms"], "p99_ms": rep["p99_ms"],
            "p99_wait_ms": rep["p99_wait_ms"], "peak_active": rep["peak_active"],
            "batched_ticks": rep["batched_ticks"], "batches_made": rep["batches_made"], "ticks": rep["ticks"]}


def _served(a, stream, plain=True):
    """The served request stream: report of the continuous-batching server
    stepping its resident scenes side by side (the faster mode on this
    stream), the same stream served in cohorts (a shared-launch batch per
    admission wave), a sweep of arrival rates in both modes when a.rates
    lists them, and the same requests' time alone in the FP64 form."""
    from metakonga_gb300 import scenes, serve
    t0 = time.perf_counter()
    reqs = scenes.served_requests(count=a.requests, seed=4)
    scs = [scenes.make_request_scene(r) for r in reqs]
    gen_s = time.perf_counter() - t0
    arrivals = serve.poisson_arrivals(len(reqs), a.rate, seed=5)
    srv = serve.Server(budget_bytes=int(a.budget_gb * 1e9), chunk=a.chunk, stream=stream.cuda_stream,
                       keep_results=True)
    for k, (r, sc) in enumerate(zip(reqs, scs)):
        srv.submit(k, sc, r["steps"], arrival=float(arrivals[k]))
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    with clk:
        srv.run()
    rep = srv.report()
    rep["clocks"] = clk.summary()
    rep["generation_s"] = gen_s
    rep["arrival_rate_per_s"] = a.rate
    rep["budget_bytes"] = int(a.budget_gb * 1e9)
    rep["chunk_steps"] = a.chunk
    rep["particles"] = [int(sc.np_) for sc in scs]
    rep["steps"] = [int(r["steps"]) for r in reqs]
    rep["kinds"] = [r["kind"] for r in reqs]
    rep["mode"] = "side_by_side"
    rep["e2e_note"] = ("latency from arrival to the downloaded result: scene upload, steps and "
                       "download through the public API (DeviceScene, xd_scene_step_many)")
    rep["cohorts"] = _serve_once(scs, reqs, a.rate, a, stream, "cohorts")
    if a.rates:
        rep["sweep"] = [_serve_once(scs, reqs, float(x), a, stream, m)
                        for x in a.rates.split(",") for m in ("cohorts", "side_by_side")]
    if plain:
        per = _fp64_alone(scs, 2, stream)
        alone_s = sum(r["steps"] * ms / 1e3 for r, ms in zip(reqs, per))
        rep["plain_fp64_alone"] = {
            "seconds_one_after_another": alone_s,
            "particle_steps_per_s": rep["particle_steps"] / alone_s,
            "method": "each request's scene alone in the FP64 form, 2 device-timed steps after one "
                      "warm-up step, times its step count; summed over requests"}
        rep["vs_plain_fp64"] = rep["particle_steps_per_s"] / (rep["particle_steps"] / alone_s)
    del rep["particles"], rep["steps"]
    return rep


def _time_batch(batch, steps, stream, barrier, world, clock_index=None):
    """Device time of `steps` batch steps (CUDA events on the launching
    stream, barriers on both sides, max over ranks); with clock_index the
    SM clocks are sampled meanwhile."""
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(clock_index) if clock_index is not None else None
    barrier()
    if clk:
        clk.__enter__()
    ev0.record(stream)
    batch.step(steps, check=False, stream=stream.cuda_stream)
    ev1.record(stream)
    barrier()
    if clk:
        clk.__exit__(None, None, None)
    ms = _max_over_ranks(ev0.elapsed_time(ev1), world)
    return ms, (clk.summary() if clk else None)


def _batch_contact_bytes(ds, sh):
    """Algorithmic bytes of one contact pass over a batch: per listed sphere
    its own state and list counts read (B_LISTED) and its force and torque
    written, plus 4 B per Verlet-list and triangle-list entry read; the
    neighbours' data count as cache-resident (0 B), the unlisted spheres are
    not visited.  Also the listed count and the mean list lengths."""
    listed = ventries = tentries = 0
    for d in ds:
        st = d.stats(sh)
        listed += st["contact_list"]
        ventries += st["verlet_entries"]
        tentries += st["triangle_entries"]
    return (listed * B_LISTED + 4 * (ventries + tentries), listed,
            ventries / max(listed, 1), tentries / max(listed, 1))


def run_batched(a):
    import numpy as np
    import torch

    from metakonga_gb300 import engine, scenes
    from metakonga_gb300._lib import call
    world, rank, local, barrier = _torch_setup()
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    peak, peak_kind = _peaks()
    specs = scenes.hopper_batch(count=a.count)
    k_med = _median_index(specs)

    # ---- the batch as generated (a loose lattice falling): beside the headline
    lattice = None
    if not a.no_lattice:
        scs_l = [scenes.hopper(**d) for d in specs]
        ds_l = [engine.DeviceScene(sc, mode=engine.MODE_MIXED) for sc in scs_l]
        b_l = engine.Batch(ds_l)
        b_l.step(a.warmup, check=True, stream=sh)
        ms_l, _ = _time_batch(b_l, a.steps, stream, barrier, world)
        n_l = sum(sc.np_ for sc in scs_l)
        lattice = {"value": world * n_l * a.steps / (ms_l / 1e3), "unit": METRIC, "ms_per_step": ms_l / a.steps,
                   "listed_fraction": sum(d.stats(sh)["contact_list"] for d in ds_l) / n_l,
                   "state": "the hoppers as generated: jittered lattices (pitch >= 2.04 r_max, no contact) "
                            f"falling, {a.warmup} warm-up steps in"}
        # the same lattices after 4,000 steps (20 ms) of falling: the lowest
        # layers piled on the cones and the floor
        b_l.step(4000, check=True, stream=sh)
        ms_f, _ = _time_batch(b_l, a.steps, stream, barrier, world)
        b_l.set_timing(True)
        b_l.step(max(3, min(a.steps, 20)), check=False, stream=sh)
        kt_f = b_l.kernel_times()
        b_l.set_timing(False)
        nf = max(kt_f["contact"][1], 1)
        lattice["fallen_4000"] = {
            "value": world * n_l * a.steps / (ms_f / 1e3), "unit": METRIC, "ms_per_step": ms_f / a.steps,
            "listed_fraction": sum(d.stats(sh)["contact_list"] for d in ds_l) / n_l,
            "pair_pass_ms": kt_f["contact"][0] / nf, "wall_pass_ms": kt_f["walls"][0] / nf,
            "advance_ms": kt_f["advance"][0] / max(kt_f["advance"][1], 1),
            "state": "the lattices after 4,000 more steps of falling at dt 5e-6"}
        b_l.close()
        for d in ds_l:
            d.close()
        del ds_l, scs_l
        torch.cuda.empty_cache()

    # ---- the headline: settled beds discharging through the opened orifice
    t0 = time.perf_counter()
    scs = _settled_hoppers(specs, a, sh)
    torch.cuda.synchronize()
    prep_s = time.perf_counter() - t0
    n_tot = sum(sc.np_ for sc in scs)
    # the autotuner on the scene at the particle-weighted median (half the
    # spheres are in larger scenes), its choice applied to every scene
    tuned = None
    tuning = dict(engine.DEFAULT_TUNING)
    tunings = [tuning] * len(scs)
    if not a.no_tune:
        # the autotuner per scene shape (particle-count octave, radius
        # spread, walls, packing: tune.shape_key) on the shape's median
        # scene, cached in a file of this run and applied to every scene of
        # the shape; the batch's launch shape and pair pass (one launch
        # serves all scenes) are those of the particle-weighted median scene
        import tempfile

        from metakonga_gb300 import tune
        cache = os.path.join(tempfile.gettempdir(), f"xdem_bench_tuning_{os.getpid()}.json")
        os.environ["XDEM_TUNE_CACHE"] = cache
        t_tune = time.perf_counter()
        groups = {}
        for k, sc in enumerate(scs):
            groups.setdefault(tune.shape_key(sc), []).append(k)
        per_shape = {}
        for key, ks in sorted(groups.items()):
            ks = sorted(ks, key=lambda k: scs[k].np_)
            rep = ks[len(ks) // 2]
            tr = tune.tune(scs[rep], steps=a.tune_steps, warm=5, store=True)
            per_shape[key] = {"scenes": len(ks), "scene": rep, "particles": int(scs[rep].np_),
                              "choice": tr["tuning"], "ms_per_step": tr["ms_per_step"],
                              "default_ms_per_step": tr["default_ms_per_step"]}
        order = np.argsort([sc.np_ for sc in scs])
        cum = np.cumsum([scs[k].np_ for k in order])
        k_w = int(order[int(np.searchsorted(cum, cum[-1] / 2))])
        launch = tune.tuned(scs[k_w])
        tunings = [dict(tune.tuned(sc), contact_threads=launch["contact_threads"],
                        contact_mode=launch["contact_mode"]) for sc in scs]
        tuning = tunings[k_w]
        try:
            os.remove(cache)
        except OSError:
            pass
        tuned = {"per_shape": per_shape, "launch_shape_scene": k_w, "launch": {
                     "contact_threads": launch["contact_threads"], "contact_mode": launch["contact_mode"]},
                 "seconds": time.perf_counter() - t_tune, "window_steps": a.tune_steps}
    ds = [engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning=t) for sc, t in zip(scs, tunings)]
    dev_bytes = sum(d.device_bytes() for d in ds)
    batch = engine.Batch(ds)
    batch.step(a.warmup, check=True, stream=sh)
    rb0 = [d.rebuilds(sh) for d in ds]
    st0 = [d.stats(sh) for d in ds]
    ms, clocks = _time_batch(batch, a.steps, stream, barrier, world, clock_index=local)
    value = world * n_tot * a.steps / (ms / 1e3)
    rb1 = [d.rebuilds(sh) for d in ds]
    st1 = [d.stats(sh) for d in ds]
    rebuilds = sum(b[0] - r[0] for r, b in zip(rb0, rb1))
    rechecks = {k: sum(y[k] - x[k] for x, y in zip(st0, st1)) / a.steps
                for k in ("fp64_decisions", "fp64_normal_forces", "fp64_slips", "fp64_wall_regions")}
    contact_bytes, listed, vlen, tlen = _batch_contact_bytes(ds, sh)
    pick = [int(i) for i in np.argsort([sc.np_ for sc in scs])[[len(scs) // 8, len(scs) // 2, -1]]]
    coord = {str(scs[i].np_): ds[i].pair_list(cap=32).shape[0] / scs[i].np_ for i in pick}

    # the kernels timed live: the same steps launched directly with CUDA
    # events around each advance and contact launch (events cannot split the
    # step graph)
    ksteps = max(3, min(a.steps, 20))
    batch.set_timing(True)
    batch.step(ksteps, check=True, stream=sh)
    kt = batch.kernel_times()
    batch.set_timing(False)
    adv_ms = kt["advance"][0] / max(kt["advance"][1], 1)
    pair_ms = kt["contact"][0] / max(kt["contact"][1], 1)
    wall_ms = kt["walls"][0] / max(kt["contact"][1], 1)   # per step (0 without a wall pass)
    con_ms = pair_ms + wall_ms
    # what a step costs beyond its two big kernels (the decision kernel, run
    # prefix, graph and conditional nodes, and the re-binnings): the most a
    # persistent batch kernel could save
    other_ms = ms / a.steps - adv_ms - con_ms
    adv_gbs = n_tot * B_ADVANCE / (adv_ms / 1e3) / 1e9
    con_gbs = contact_bytes / (con_ms / 1e3) / 1e9
    adv_traffic = _traffic_from_profiles("advance_batch_hopper.md", "traffic_bytes_per_particle")
    con_traffic = _traffic_from_profiles("contact_mixed_hopper_settled.md", "traffic_bytes_per_listed_sphere")
    kernels = {
        "advance": {"kernel": "k_batch_advance<1> (velocity-Verlet kick and drift, contact view and skin test of "
                              "every scene's spheres in one launch)",
                    "avg_launch_ms": adv_ms, "bytes": n_tot * B_ADVANCE, "bytes_per_particle": B_ADVANCE,
                    "achieved": adv_gbs, "frac": adv_gbs / peak,
                    "traffic": adv_traffic * n_tot if adv_traffic else None},
        "contact": {"kernel": "k_batch_contact<1> + <2> (every scene's listed spheres: the cooperative pair pass "
                              "over the Verlet lists in one launch, then the wall pass over the listed spheres "
                              "with planes or triangles in reach in another)",
                    "avg_launch_ms": con_ms, "pair_pass_ms": pair_ms, "wall_pass_ms": wall_ms,
                    "bytes": contact_bytes, "listed": listed,
                    "bytes_per_listed_sphere": contact_bytes / max(listed, 1),
                    "mean_verlet_entries": vlen, "mean_triangle_entries": tlen,
                    "achieved": con_gbs, "frac": con_gbs / peak,
                    "traffic": con_traffic * listed if con_traffic else None},
    }
    dom = "contact" if con_ms >= adv_ms else "advance"
    dk = kernels[dom]
    roof = {"bound": "hbm", "kernel": dk["kernel"], "achieved": dk["achieved"], "peak": peak, "unit": "GB/s",
            "frac": dk["frac"], "peak_kind": peak_kind, "traffic": dk["traffic"], "avg_launch_ms": dk["avg_launch_ms"],
            "launches_timed": kt[dom][1],
            "algorithmic_bytes_per_launch": dk["bytes"],
            "workload": f"the {len(scs)} settled hoppers ({n_tot:,} spheres); {ksteps} steps with direct "
                        "launches after the timed ones",
            "kernels": kernels,
            "traffic_note": "DRAM bytes per unit of one ncu-captured launch (profiles/advance_batch_hopper.md per "
                            "sphere, profiles/contact_mixed_hopper_settled.md per listed sphere, pair and wall "
                            "passes) times the units here"}
    # per step: advance, decision, run prefix and contact over all scenes; per
    # call the finish and each scene's body-reaction sum; per re-binning its
    # kernels and its group's decision kernel
    walls_pass = 1 if tunings[0].get("contact_mode", 1) == 1 else 0   # the cooperative pass's wall launch
    launches = ((4 + walls_pass) * a.steps + 1 + sum(1 for sc in scs if sc.ntri)
                + sum((b[0] - r[0]) * (b[1] + 1) for r, b in zip(rb0, rb1)))

    # e2e: every scene's state uploaded from pinned host memory, K steps, the
    # state downloaded; the downloaded state is the next upload's input
    keys = ("pos", "vel", "acc", "omega", "alpha")
    host = []
    for d, sc in zip(ds, scs):
        st = d.download(sh)
        # one pinned block per scene, the arrays back to back in the order the
        # library stages them (pos, vel, acc, omega, alpha, mass, inertia): the
        # upload and the download then go as one copy each
        n = sc.np_
        block = torch.empty(18 * n, dtype=torch.float64).pin_memory()
        h, off = {}, 0
        for k, w in (("pos", 4), ("vel", 3), ("acc", 3), ("omega", 3), ("alpha", 3), ("mass", 1), ("inertia", 1)):
            h[k] = block[off:off + w * n]
            src = st[k] if k in keys else getattr(sc, k)
            h[k].copy_(torch.from_numpy(np.ascontiguousarray(src).reshape(-1)))
            off += w * n
        for k in ("force", "moment"):
            h[k] = torch.from_numpy(np.ascontiguousarray(getattr(sc, k))).pin_memory()
        host.append(h)
    h2d = sum(sum(h[k].numel() * 8 for k in keys + ("mass", "inertia")) for h in host)
    d2h = sum(sum(h[k].numel() * 8 for k in keys) for h in host)

    def e2e_job():
        # copies queued on the stream (pinned buffers), one wait at the end
        for d, h in zip(ds, host):
            call("xd_scene_upload_async", d.handle, *[h[k].data_ptr() for k in
                                                      ("pos", "vel", "acc", "omega", "alpha", "force",
                                                       "moment", "mass", "inertia")], sh)
        batch.step(a.steps, check=False, stream=sh)
        for d, h in zip(ds, host):
            call("xd_scene_download_async", d.handle, *[h[k].data_ptr() for k in keys], None, None, sh)
        torch.cuda.current_stream().synchronize()
        stream.synchronize()

    barrier()
    t1 = time.perf_counter()
    e2e_job()
    barrier()
    e2e_s = _max_over_ranks(time.perf_counter() - t1, world)
    e2e_value = world * n_tot * a.steps / e2e_s
    batch.close()
    for d in ds:
        d.close()
    del host
    torch.cuda.empty_cache()

    plain = None
    if not a.no_plain:
        psteps = 2
        per = _fp64_alone(scs, psteps, stream)
        fp64_ms = sum(per)
        plain = {"value": world * n_tot / (fp64_ms / 1e3), "unit": METRIC,
                 "ms_per_batch_step": fp64_ms,
                 "method": "each settled scene alone in the FP64 form (the reference's algorithm: 128^3 grid "
                           "of 2 x max(r, triangle circumradius) cells, re-sorted every step), one "
                           f"warm-up step then {psteps} device-timed steps; ms summed over scenes",
                 "ratio": value / (world * n_tot / (fp64_ms / 1e3))}
        per_g = _fp64_alone(scs, psteps, stream, own_grid=True)
        fp64g_ms = sum(per_g)
        plain["own_grid"] = {
            "value": world * n_tot / (fp64g_ms / 1e3), "unit": METRIC, "ms_per_batch_step": fp64g_ms,
            "method": "the same, with the particles on a grid of their own (cells of the largest diameter, "
                      "power-of-two dimensions holding the bed unwrapped) and the triangles on the reference's "
                      "(xd_scene_set_particle_grid): the FP64 form on particle cells of the mixed form's size",
            "ratio": value / (world * n_tot / (fp64g_ms / 1e3))}

    # FP64 check on the median scene's settled bed
    check = _fp64_check(scs[k_med], squeeze=1.0, spin=False)
    check["scene"] = k_med
    # the batch with the default tuning, for the autotuner's gain
    if tuned is not None:
        if any(t != engine.DEFAULT_TUNING for t in tunings):
            ds0 = [engine.DeviceScene(sc, mode=engine.MODE_MIXED) for sc in scs]
            b0 = engine.Batch(ds0)
            b0.step(a.warmup, check=True, stream=sh)
            ms0, _ = _time_batch(b0, a.steps, stream, barrier, world)
            b0.close()
            for d in ds0:
                d.close()
            del ds0
            torch.cuda.empty_cache()
            tuned["batch_default_ms_per_step"] = ms0 / a.steps
        else:
            tuned["batch_default_ms_per_step"] = ms / a.steps
        tuned["batch_ms_per_step"] = ms / a.steps
        tuned["gain"] = tuned["batch_default_ms_per_step"] / tuned["batch_ms_per_step"]
    box_roof, box = _box_roofline(a, stream, barrier, world, local) if not a.no_box else (None, None)
    settle = _settle_small(stream, cpu=not a.no_cpu_baseline) if rank == 0 and not a.no_box else None
    if box:
        box["roofline"] = box_roof
    drum = _drum(a, stream) if not a.no_drum and rank == 0 else None
    served = _served(a, stream, plain=not a.no_plain) if rank == 0 and not a.no_served else None

    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        csteps = a.cpu_steps or 20
        vals, times = cpu_baseline([("scene", scs[k_med])], csteps, samples=1)
        cpu = {"value": vals[0], "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"{csteps} steps of scene {k_med} of the batch ({scs[k_med].np_} spheres, the median; "
                         f"its settled bed as timed here), reference CPU path (restated, single thread, "
                         f"polygon contacts included), {times[0]:.1f} s",
               "host": host_cpu()}
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded MT19937 scenes: settled beds in cones of triangles)",
        "config": {"workload": BATCH_WORKLOAD, "scenes": len(scs), "particles": n_tot,
                   "particles_min": min(sc.np_ for sc in scs), "particles_max": max(sc.np_ for sc in scs),
                   "triangles_per_scene": int(scs[0].ntri), "dt": 5e-6, "mode": "mixed",
                   "state": (f"settled beds discharging: each hopper filled as a lattice with its orifice gated, "
                             f"settled by {a.prep_steps} steps of {a.prep_dt:g} s in the mixed form "
                             f"({prep_s:.0f} s, untimed), the gate then opened; {a.warmup} warm-up steps"),
                   "listed_fraction": listed / n_tot,
                   "mean_coordination": coord,
                   "fp64_rechecks_per_step": rechecks,
                   "grid": "one grid per scene sized to its cone, cell 2 r_max + skin",
                   "stepping": ("xd_batch: CUDA graphs of one or four batch steps -- one advance and one contact "
                                "launch over all scenes, each scene's re-binning behind conditional nodes"),
                   "l2": "batch state > L2 (no flush)", "device_bytes": dev_bytes,
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d / a.steps,
                "d2h_bytes_per_step": d2h / a.steps, "h2d_bytes_per_job": h2d, "d2h_bytes_per_job": d2h,
                "job": f"upload all {len(scs)} states from pinned host memory, {a.steps} steps, download"},
        "gpu_launches": launches,
        "cell_rebinnings_in_timed_steps": rebuilds,
        "autotune": tuned,
        "step_beyond_kernels_ms": {"value": other_ms, "of_step": other_ms / (ms / a.steps),
                                   "note": "ms per batch step minus the advance and contact launches' live "
                                           "times: re-binnings, the decision kernel, run prefix, graph and "
                                           "conditional nodes -- the most a persistent kernel could save"},
        "lattice_start": lattice,
        "plain_fp64": plain,
        "plain_fp64_own_grid": plain["own_grid"] if plain else None,
        "fp64_check": check,
        "roofline": roof,
        "single_scene_box": box,
        "settle_8000": settle,
        "drum": drum,
        "served": served,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_served(a):
    import torch
    world, rank, local, barrier = _torch_setup()
    stream = torch.cuda.Stream()
    rep = _served(a, stream, plain=not a.no_plain)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": rep["particle_steps_per_s"], "unit": METRIC, "n_gpus": world,
        "steps": a.requests, "warmup": 0, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded MT19937 request stream)",
        "config": {"workload": SERVED_WORKLOAD, "requests": a.requests, "rate_per_s": a.rate,
                   "budget_gb": a.budget_gb, "chunk": a.chunk, "mode": "mixed"},
        "e2e": {"value": rep["particle_steps_per_s"], "unit": METRIC,
                "note": "the served value is end to end (upload, steps, download per request)"},
        "p50_ms": rep["p50_ms"], "p99_ms": rep["p99_ms"], "served": rep,
        "clocks": rep["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_drum(a):
    """The rotating drum on its own (the batched line carries it as "drum")."""
    import torch
    world, rank, local, barrier = _torch_setup()
    stream = torch.cuda.Stream()
    clk = ClockSampler(local)
    with clk:
        d = _drum(a, stream, steps=a.steps, warmup=a.warmup, plain=not a.no_plain)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": d["value"], "unit": METRIC, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": d["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded MT19937 jittered FCC lattice in a cylinder of triangles)",
        "config": {"workload": "rotating_drum_500k", "particles": 500_000, "triangles": 20_480,
                   "dt": 5e-6, "mode": "mixed", "l2": "state > L2 (no flush)"},
        "drum": d, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def _settled_hopper(n, seed=5, prep_steps=5000, prep_dt=4e-5):
    """One hopper of n spheres as a settled bed with its orifice open (the
    batch's preparation), cached in the temp directory so that a profiler's
    run of this workload loads it instead of launching the preparation."""
    import tempfile

    import numpy as np

    from metakonga_gb300 import prepare, scenes
    sc = scenes.hopper(n=n, seed=seed, gate=True)
    path = os.path.join(tempfile.gettempdir(), f"xdem_hopper_settled_{n}_seed{seed}_{prep_steps}.npz")
    keys = ("pos", "vel", "acc", "omega", "alpha")
    try:
        z = np.load(path)
        for k in keys:
            getattr(sc, k)[:] = z[k]
    except (OSError, KeyError, ValueError):
        prepare.settle(sc, prep_steps, dt=prep_dt)
        try:
            np.savez(path, **{k: getattr(sc, k) for k in keys})
        except OSError:
            pass
    prepare.open_gates(sc)
    return sc


def run_hopper(a):
    """One settled hopper (a.hopper_n spheres, the batch's preparation) in
    the mixed form, its contact pass timed per kernel: the workload the
    contact-pass profiles are taken on."""
    import torch

    from metakonga_gb300 import engine
    world, rank, local, barrier = _torch_setup()
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    sc = _settled_hopper(a.hopper_n, prep_steps=a.prep_steps, prep_dt=a.prep_dt)
    d = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    d.step(a.warmup, check=True, stream=sh)
    st0 = d.stats(sh)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local)
    with clk:
        e0.record(stream)
        d.step(a.steps, check=False, stream=sh)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    st1 = d.stats(sh)
    d.set_timing(True)
    d.step(a.steps, check=False, stream=sh)
    ph = d.phase_times()
    d.set_timing(False)
    d.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": world * sc.np_ * a.steps / (ms / 1e3), "unit": METRIC, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded MT19937 hopper, settled with its orifice gated, then opened)",
        "config": {"workload": f"hopper_settled_{sc.np_}", "particles": int(sc.np_), "triangles": int(sc.ntri),
                   "dt": 5e-6, "mode": "mixed", "l2": "state < L2 (a single-scene profile case)"},
        "phases_ms": {k: v[0] / max(v[1], 1) for k, v in ph.items() if v[1]},
        "per_step": {k: (st1[k] - st0[k]) / a.steps for k in ("fp64_decisions", "fp64_normal_forces",
                                                              "fp64_slips", "fp64_wall_regions")},
        "listed": st1["contact_list"], "listed_with_walls": st1["listed_with_triangles"],
        "verlet_entries": st1["verlet_entries"], "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "batched":
        run_batched(a)
    elif a.workload == "served":
        run_served(a)
    elif a.workload == "drum":
        run_drum(a)
    elif a.workload == "hopper":
        run_hopper(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
