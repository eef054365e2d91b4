"""Benchmark of the GB300 PlayRho world step.

Default workload: 4096 independent worlds (body counts log-uniform in [16, 2048],
half box pyramids, half piles of disks and 3-8-gons, seed 1; ~1.6 M bodies)
advanced together in one CUDA-graph step (dt 1/60, 8/3 iterations, float32).

A body-step is one awake dynamic body advanced one step (the device counts the
dynamic bodies of awake islands; sleeping bodies are not counted).  Every arm
runs the same untimed steps first (settling, autotuning, warm-up), so all of
them time the same state of the simulation.

  value : body-steps/s of the batched step, inputs resident in HBM, device time
          from CUDA events the captured step graph records around its phases
  e2e   : the same metric through the C ABI with host buffers: every step
          uploads the body states from pinned host memory, steps, and reads them
          back, all inside the host-timed region
  roofline : the Gauss-Seidel sweep kernel (the dominant phase), algorithmic
          bytes per launch over its live CUDA-event duration vs measured HBM peak
  cpu_baseline : the reference's own step (its library built from the staged
          sources; the oracle port where they are absent) on one host core, on
          every 64th world

``--impl reference`` times the reference's CPU step on all host cores (one
process per core, every world of the workload) and prints the same metric.
Multi-GPU (torchrun): each rank advances its own copy of the batch (worlds are
independent; no collective on the data path), scaling "weak".
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched body-steps/s"
UNIT = "body-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--worlds", type=int, default=4096)
    p.add_argument("--settle", type=int, default=None,
                   help="untimed steps that bring the scenes to their contact-rich state (default per workload)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the StepAdjoint measurement")
    p.add_argument("--no-toi", action="store_true", help="skip the time-of-impact (doToi) measurement")
    p.add_argument("--toi", action="store_true",
                   help="run the workload's timed steps with the time-of-impact phase on (doToi = 1)")
    p.add_argument("--sweeps", default="auto", choices=["auto", "grid", "per_world"],
                   help="scheduling of the colour sweeps (auto: one CTA per world for >= 64 worlds)")
    p.add_argument("--kernels-only", action="store_true",
                   help="only the warm-up and timed steps (for a profiler launch list)")
    p.add_argument("--workload", default="batched", choices=list(WORKLOADS),
                   help="batched: the headline batch (default); world100k: one world of 100,000 shapes in a "
                        "1000 m box; chains256: 256 worlds of 8,000 free shapes + 64 revolute chains of 32 links; "
                        "bullets1024: 1024 worlds of 40 fast shapes in closed boxes with the time-of-impact phase")
    return p.parse_args()


# name -> (description, step configuration overrides, default settling steps)
WORKLOADS = {
    "batched": ("batched worlds: {n} worlds, log-uniform 16..2048 bodies, pyramids + piles, seed 1", {}, 240),
    "world100k": ("one world: 100,000 shapes (disks + 3..8-gons) in a 1000 m box, seed 0", {}, 60),
    "chains256": ("{n} worlds x (8,000 free shapes + 64 chains x 32 links on revolute joints), seed 3",
                  {"deltaTime": 1.0 / 120.0, "regVelocityIters": 10, "regPositionIters": 4}, 120),
    "bullets1024": ("{n} worlds x 40 fast disks and 3..8-gons (60..180 m/s, half bullets) in a closed 30 m box, "
                    "seed 9, time-of-impact phase on", {"doToi": 1}, 3),
}


def workload(args):
    from playrho_gb300 import scenes

    if args.workload == "world100k":
        return [scenes.large_box(100_000, 1000.0, seed=0)]
    if args.workload == "chains256":
        rng = np.random.default_rng(3)
        n = args.worlds if args.worlds != 4096 else 256
        return [scenes.chains_world(rng) for _ in range(n)]
    if args.workload == "bullets1024":
        rng = np.random.default_rng(9)
        n = args.worlds if args.worlds != 4096 else 1024
        return [scenes.bullets(40, rng, size=15.0) for _ in range(n)]
    return scenes.batched_worlds(args.worlds, seed=1)


def dist_setup(args):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        td.init_process_group(backend, init_method="env://")
        dist = td
    return rank, world, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([float(v)], device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """Samples SM clocks and throttle reasons while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = []
        reasons = set()
        smax = None
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax = float(r[1])
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                for n, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(n)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sweep_bytes(stats, conf, n_bodies_solved):
    """Algorithmic bytes of one Gauss-Seidel sweep launch (warm start, velocity and
    position iterations, integration, impulse store) for the active constraints."""
    nc = stats["activeConstraints"]
    iv = conf.regVelocityIters
    ip = stats["sumPosIters"] / max(1, stats["islandsFound"])  # mean position iterations per island
    per_contact = 160 + 240 * iv + 160 * ip + 32
    return nc * per_contact + n_bodies_solved * 52


def update_bytes(st, worlds) -> float:
    """Algorithmic bytes of the post-solve contact maintenance phase: k_synchronize
    (each shape's body and flags, both transforms and its box read, the moved flag
    written: 60 B; its vertices read for the swept box: 12 + 16 nv B), then
    k_update_contacts over the contacts of moved bodies (every live contact's flags
    and body ids read: 12 B; each contact updated reads its proxy ids and old
    manifold and writes the new manifold, flags and phase tag: 8 + 60 + 60 + 4 + 8
    = 140 B; each shape's record and vertices read once more: 12 + 16 nv B, and
    each body's transform and flags: 20 B)."""
    n_shapes = sum(w.n_shapes for w in worlds)
    n_verts = sum(int(w.shape_nv.sum()) for w in worlds)
    n_bodies = sum(w.n_bodies for w in worlds)
    shape_bytes = 12 * n_shapes + 16 * n_verts
    return (60 * n_shapes + 2 * shape_bytes + 20 * n_bodies + 12 * st["liveContacts"]
            + 140 * st["contactsUpdated"])


def profile_figure(name: str, key: str):
    """A figure (`key: value` line) of an ncu summary under profiles/."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":")[1])
    except OSError:
        pass
    return None


# prgpu_autotune times 22 candidate schedules (the grid-wide one, 3 staging sizes
# x 5 warp-world limits, then 2 warp-world limits x 3 group-world limits), then
# the 3 fastest once more, each timing over one capturing step plus the steps
# asked for; those steps advance the batch like any other.
AUTOTUNE_CANDIDATES = 22 + 3
AUTOTUNE_STEPS = 2


def steps_before_timing(args) -> int:
    """Steps every arm runs on the workload before its timed steps: the settling
    steps, the autotuner's steps and the warm-up steps, so that all arms time the
    same state of the simulation."""
    tune = AUTOTUNE_CANDIDATES * (1 + AUTOTUNE_STEPS) if args.sweeps == "auto" else 0
    return args.settle + tune + max(3, args.warmup)


def balanced_shares(worlds, parts):
    """Splits world indices into `parts` shares of about equal body counts
    (largest world first into the lightest share)."""
    order = sorted(range(len(worlds)), key=lambda i: -worlds[i].n_bodies)
    shares = [[] for _ in range(parts)]
    load = [0] * parts
    for i in order:
        k = load.index(min(load))
        shares[k].append(i)
        load[k] += worlds[i].n_bodies
    return [sorted(s) for s in shares if s]


def _port_worker(idx, workload_args, pre, steps, overrides, barrier, out):
    """Oracle-port process: builds its share of the workload's worlds, runs the
    untimed steps, waits for the other processes, then times its steps."""
    sys.path.insert(0, ROOT)
    from oracle import oracle

    worlds = workload(workload_args)
    mine = [(oracle.OracleWorld(worlds[i]), worlds[i].body_type == 2) for i in idx]
    for _ in range(pre):
        for o, _dyn in mine:
            o.step(**overrides)
    barrier.wait()
    seconds, body_steps = 0.0, 0
    for _ in range(steps):
        for o, dyn in mine:
            body_steps += int(((o.bodies()["awake"] != 0) & dyn).sum())
            t0 = time.perf_counter()
            o.step(**overrides)
            seconds += time.perf_counter() - t0
    out.put((seconds, body_steps))


def cpu_step_runs(args, worlds, idx_shares, pre, steps, overrides):
    """Times the reference's CPU step on shares of the workload, one process per
    share, all processes starting their timed steps together.  Uses the
    reference's own library (oracle/_ref/ref_bench_f32, built from the staged
    reference sources) where it can be built, else the oracle port.  Returns
    (kind, [(seconds, awake body-steps), ...])."""
    from oracle import refdriver

    if refdriver.staged():
        try:
            exe = refdriver.ensure_bench_built()
        except Exception as e:  # the reference does not build on this host: use the port
            print(f"reference bench driver not built ({e}); timing the oracle port", file=sys.stderr)
            exe = None
        if exe:
            from playrho_gb300 import scenes

            conf = "".join(f"conf {k} {float(v)!r}\n" for k, v in overrides.items())
            procs = []
            for share in idx_shares:
                p = subprocess.Popen([exe], stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True)
                text = "".join("world\n" + scenes.scene_text(worlds[i]) for i in share)
                p.stdin.write(text + conf + f"run {pre}\nready\n")
                p.stdin.flush()
                procs.append(p)
            for p in procs:
                line = p.stdout.readline().split()
                if not line or line[0] != "ready":
                    raise RuntimeError("reference bench driver failed")
            for p in procs:
                p.stdin.write(f"go\ntime {steps}\n")
                p.stdin.flush()
            res = []
            for p in procs:
                r = p.stdout.readline().split()
                p.stdin.close()
                p.wait()
                res.append((float(r[1]), int(r[2])))
            return "reference", res
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(len(idx_shares))
    q = ctx.Queue()
    wargs = argparse.Namespace(**{k: getattr(args, k) for k in ("workload", "worlds")})
    procs = [ctx.Process(target=_port_worker, args=(s, wargs, pre, steps, overrides, barrier, q)) for s in idx_shares]
    for p in procs:
        p.start()
    res = [q.get() for _ in procs]
    for p in procs:
        p.join()
    return "port", res


def cpu_sample_desc(kind, n_worlds, n_sample, procs, pre, steps):
    what = ("the reference's library (Step over each world)" if kind == "reference"
            else "the oracle port (bit-exact restatement of the reference step), the reference sources being absent")
    return (f"{n_sample} of {n_worlds} worlds on {procs} process{'es' if procs > 1 else ''}, {steps} timed steps "
            f"after {pre} untimed ones (the GPU arm's settling, autotuning and warm-up steps), {what}; "
            f"body-steps = awake dynamic bodies before each step")


def run_reference(args, rank):
    """The reference's CPU step on the host's cores: the same worlds, the same
    untimed steps before timing, the same metric (awake body-steps/s).  Under
    torchrun only rank 0 runs it."""
    if rank != 0:
        return
    desc, overrides, settle = WORKLOADS[args.workload]
    if args.settle is None:
        args.settle = settle
    if args.toi:
        overrides = dict(overrides, doToi=1)
    worlds = workload(args)
    pre = steps_before_timing(args)
    cores = os.cpu_count() or 1
    shares = balanced_shares(worlds, cores)
    kind, res = cpu_step_runs(args, worlds, shares, pre, args.steps, overrides)
    tmax = max(r[0] for r in res)
    body_steps = sum(r[1] for r in res)
    value = body_steps / tmax
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": tmax / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic",
           "config": {"workload": desc.format(n=len(worlds)), "worlds": len(worlds),
                      "dynamic_bodies": sum(w.n_dynamic() for w in worlds),
                      "awake_body_steps_per_step": body_steps / args.steps,
                      "steps_before_timing": pre, "processes": len(shares)},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": len(shares), "kind": kind,
                            "sample": cpu_sample_desc(kind, len(worlds), len(worlds), len(shares), pre,
                                                      args.steps)},
           # one core's figure: each process's own rate over its share of the worlds
           "single_thread": {"value": statistics.mean(r[1] / r[0] for r in res if r[0] > 0), "unit": UNIT,
                             "cores": 1, "sample": f"mean over the {len(shares)} processes of each one's "
                                                   "awake body-steps over its own timed steps"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_ours(args, rank, world_size, local, dist):
    from playrho_gb300 import build, gpu

    build.build()
    worlds = workload(args)
    desc, overrides, settle = WORKLOADS[args.workload]
    if args.toi:
        overrides = dict(overrides, doToi=1)
        desc += ", time-of-impact phase on"
    if args.settle is None:
        args.settle = settle
    n_dyn = sum(int((w.body_type == 2).sum()) for w in worlds)
    batch = gpu.GpuBatch(worlds, device=local)
    batch.set_sweep_mode(args.sweeps)
    conf = gpu.default_conf(**overrides)
    # Scene preparation: advance the batch `settle` steps (piles land, pyramids take
    # their load) so the measured steps are the contact-rich middle of the run,
    # then W warm-up steps.  The first step creates every proxy and contact, as
    # the reference's does.
    batch.step_n(args.settle, conf)
    schedule = None
    if args.sweeps == "auto":
        # the autotuner times each candidate sweep schedule on the settled batch
        # (those steps advance it, like settling steps) and keeps the fastest
        schedule = batch.autotune(AUTOTUNE_STEPS, conf)
    for _ in range(max(3, args.warmup)):
        batch.step_n(1, conf)
    barrier(dist)
    step_ms, phases = [], []
    nvtx = nvtx_ranges()
    body_steps0 = batch.body_steps()
    with Clocks(local) as clk:
        nvtx[0]("timed")  # a profiler can select the timed steps by this range
        for _ in range(args.steps):
            if conf.doToi:
                # the TOI loop syncs with the host between rounds: host clock over the whole step
                t = time.perf_counter()
                batch.step_n(1, conf)
                ms = (time.perf_counter() - t) * 1e3
                ph = batch.last_step_phase_ms()
                ph["toi"] = ms - ph["step"]
                ph["step"] = ms
            else:
                batch.step_async(1, conf)
                ph = batch.last_step_phase_ms()
            phases.append(ph)
            step_ms.append(ph["step"])
        batch.synchronize()
        nvtx[1]()
    barrier(dist)
    # body-steps: the dynamic bodies of awake islands in each timed step, counted
    # on the device (sleeping bodies are not counted)
    timed_body_steps = batch.body_steps() - body_steps0
    total_s = max_over_ranks(dist, sum(step_ms) / 1e3)
    value = world_size * timed_body_steps / total_s
    # statistics of one more step (outside the timed region) for the roofline bytes
    _, st = batch.step_profiled(conf)
    sweeps_ms = statistics.mean(p["sweeps"] for p in phases)
    n_solved = st["bodiesSolved"]  # bodies integrated by the sweep kernel in that step
    bytes_sweep = sweep_bytes(st, conf, n_solved)
    peak, peak_kind = measured_peaks()
    achieved = bytes_sweep / (sweeps_ms / 1e3) / 1e9

    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "kernels_only": True,
                              "ms_per_step": statistics.mean(step_ms), "sweeps": batch.sweep_mode(),
                              "warp_world_max_bodies": batch.warp_world_max_bodies(), "autotune": schedule,
                              "phase_ms": {k: statistics.mean(p[k] for p in phases) for k in phases[0]}}))
        return
    # e2e through the C ABI with host buffers (pinned), copies inside the timed region
    import torch

    nb = batch.n_bodies
    pos_h = torch.empty((nb, 3), dtype=torch.float32, pin_memory=True)
    vel_h = torch.empty((nb, 3), dtype=torch.float32, pin_memory=True)
    b0 = batch.bodies()
    pos_h.numpy()[:] = b0["pos"]
    vel_h.numpy()[:] = b0["vel"]
    lib = batch.lib
    import ctypes

    pp, vp = ctypes.c_void_p(pos_h.data_ptr()), ctypes.c_void_p(vel_h.data_ptr())
    e2e_steps = max(3, args.steps // 2)
    barrier(dist)
    e2e_bs0 = batch.body_steps()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch._check(lib.prgpu_upload_body_states(batch.h, 0, nb, pp, vp), "upload")
        batch._check(lib.prgpu_step_n(batch.h, ctypes.byref(conf), 1), "step")
        batch._check(lib.prgpu_download_bodies(batch.h, pp, vp, None, None, None, None), "download")
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e_value = world_size * (batch.body_steps() - e2e_bs0) / e2e_s

    # The plain single-world GPU step on a sample of the same worlds in the same
    # state (one world per handle and per call): each sampled world is rebuilt from
    # the batch's current bodies (positions, velocities, sleep), then 3 untimed
    # steps find its contacts again and restore warm starting before 10 timed ones.
    plain = None
    if rank == 0:
        from playrho_gb300 import scenes

        every = max(1, len(worlds) // 48)
        idx = list(range(0, len(worlds), every))[:48]
        bnow = batch.bodies()
        singles = []
        for i in idx:
            lo, hi = int(batch.body_base[i]), int(batch.body_base[i + 1])
            singles.append(gpu.GpuBatch([scenes.rebase(worlds[i], bnow["pos"][lo:hi], bnow["vel"][lo:hi],
                                                       bnow["local_center"][lo:hi], bnow["awake"][lo:hi])],
                                        device=local))
        for s in singles:
            s.step_n(3, conf)
        bs0 = sum(s.body_steps() for s in singles)
        t0 = time.perf_counter()
        for _ in range(10):
            for s in singles:
                s.step_n(1, conf)
        plain_dt = time.perf_counter() - t0
        plain = (sum(s.body_steps() for s in singles) - bs0) / plain_dt
        for s in singles:
            s.close()

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        # the reference's step on one core, on every 64th world of the workload, after
        # the same untimed steps as the timed region of this arm
        sample = list(range(0, len(worlds), 64 if len(worlds) >= 256 else max(1, len(worlds) // 4)))
        pre = steps_before_timing(args)
        kind, res = cpu_step_runs(args, worlds, [sample], pre, args.steps, overrides)
        cpu = {"value": res[0][1] / res[0][0], "unit": UNIT, "cores": 1, "kind": kind,
               "sample": cpu_sample_desc(kind, len(worlds), len(sample), 1, pre, args.steps)}
    clocks = clk.summary()
    # DRAM bytes of one solver launch on this workload, from the ncu capture
    # summarised in profiles/ (a profiler run is never part of the bench)
    traffic = upd_traffic = None
    if args.workload == "batched" and args.worlds == 4096:  # the captures cover the default batch only
        traffic = profile_figure("k_world_solve_1024_full.md", "dram_bytes_per_launch")
        upd_traffic = profile_figure("k_update_contacts_4096.md", "dram_bytes_per_phase")
    upd_ms = statistics.mean(p["sync_update"] for p in phases)
    bytes_upd = update_bytes(st, worlds)
    achieved_upd = bytes_upd / (upd_ms / 1e3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc.format(n=len(worlds)), "worlds": len(worlds), "dynamic_bodies": n_dyn,
                   "awake_bodies": timed_body_steps / args.steps,
                   "asleep_bodies": n_dyn - timed_body_steps / args.steps,
                   "body_step": "one awake dynamic body advanced one step (sleeping bodies not counted)",
                   "dt": f"1/{round(1.0 / conf.deltaTime)}",
                   "iterations": f"{conf.regVelocityIters}/{conf.regPositionIters}",
                   "parallelism": f"replicas x{world_size}",
                   "settle_steps": args.settle, "steps_before_timing": steps_before_timing(args),
                   "l2": "working set > 129 MB L2 (no flush needed)",
                   "live_contacts": st["liveContacts"], "active_constraints": st["activeConstraints"],
                   "colours": st["colours"], "serial_constraints": st["serialConstraints"],
                   "schedule": {"sweeps": batch.sweep_mode(), "warp_world_max_bodies": batch.warp_world_max_bodies(),
                                "group_world_max_bodies": batch.group_world_max_bodies(),
                                "stage_bytes": batch.stage_bytes(), "autotuned": schedule is not None}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "kernel": ("k_world_solve (per-world colouring, constraint build and Gauss-Seidel sweeps)"
                                if batch.sweep_mode() == "per_world" else
                                "k_solve (Gauss-Seidel colour sweeps, cooperative grid)"),
                     "peak_source": peak_kind, "launch_ms": sweeps_ms, "algorithmic_bytes": bytes_sweep},
        "update_roofline": {"bound": "hbm", "achieved": achieved_upd, "peak": peak, "unit": "GB/s",
                            "frac": achieved_upd / peak, "traffic": upd_traffic,
                            "kernel": "post-solve contact maintenance (k_synchronize, then k_update_contacts "
                                      "over the contacts of moved bodies)",
                            "peak_source": peak_kind, "phase_ms": upd_ms, "algorithmic_bytes": bytes_upd,
                            "contacts_updated": st["contactsUpdated"]},
        "phase_ms": {k: statistics.mean(p[k] for p in phases) for k in phases[0]},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nb * 24, "d2h_bytes_per_step": nb * 24},
        "plain_single_world_gpu": {"value": plain, "unit": UNIT,
                                   "batched_over_plain": (value / plain) if plain else None},
        "gpu_launches": None,
        "clocks": clocks,
    }
    out["gpu_launches"] = launches_per_step(batch) * args.steps
    if args.workload == "batched" and not args.no_toi:
        out["toi"] = toi_bench(args, batch, overrides, local)
    if args.workload == "batched" and not args.no_adjoint:
        out["adjoint"] = adjoint_bench(local)
    if args.workload == "chains256" and not args.no_adjoint:
        batch.close()
        out["adjoint"] = adjoint_window_bench(worlds, conf, local, args.settle)
    print(json.dumps(out), flush=True)


def _timed_steps(batch, conf, steps):
    """Host-clock seconds of `steps` synchronous steps and their statistics."""
    stats = []
    t0 = time.perf_counter()
    for _ in range(steps):
        stats.append(batch.step(conf))
    return time.perf_counter() - t0, stats


def toi_bench(args, batch, overrides, device, steps=10, n_bullet_worlds=1024, bullet_steps=20):
    """The step with the time-of-impact phase on (StepConf::doToi, the reference's
    default).  (1) The settled headline batch: body-steps/s with and without the
    TOI phase, its rounds and events per step.  (2) A TOI-heavy batch: 1024 worlds
    of 40 fast disks and polygons (60-180 m/s, half of them bullets) in closed
    15 m boxes, with the reference's step on one core on a sample of it beside it.
    Host clock around synchronous prgpu_step calls (the TOI loop reads the device
    counters between rounds, so these steps are not graph replays).  Body-steps
    count awake dynamic bodies."""
    from playrho_gb300 import gpu, scenes

    off = gpu.default_conf(**overrides)
    on = gpu.default_conf(**overrides, doToi=1)
    for c in (on, off):
        _timed_steps(batch, c, 2)
    bs0 = batch.body_steps()
    t_on, st_on = _timed_steps(batch, on, steps)
    bs_on = batch.body_steps() - bs0
    t_off, _ = _timed_steps(batch, off, steps)
    rounds = [s["toiRounds"] for s in st_on]
    headline = {
        "value": bs_on / t_on, "unit": UNIT, "ms_per_step": t_on / steps * 1e3,
        "without_toi_ms_per_step": t_off / steps * 1e3,
        "toi_rounds_per_step": statistics.mean(rounds), "toi_events_per_step":
            statistics.mean(s["toiContactsFound"] for s in st_on),
        "toi_computed_per_step": statistics.mean(s["toiContactsUpdatedToi"] for s in st_on)}
    rng = np.random.default_rng(9)
    worlds = [scenes.bullets(40, rng, size=15.0) for _ in range(n_bullet_worlds)]
    g = gpu.GpuBatch(worlds, device=device)
    _timed_steps(g, on, 3)
    bs0 = g.body_steps()
    t_b, st_b = _timed_steps(g, on, bullet_steps)
    bs_b = g.body_steps() - bs0
    g.close()
    targs = argparse.Namespace(workload="bullets1024", worlds=n_bullet_worlds)
    kind, res = cpu_step_runs(targs, worlds, [list(range(16))], 3, bullet_steps, {"doToi": 1})
    bullets = {
        "value": bs_b / t_b, "unit": UNIT, "ms_per_step": t_b / bullet_steps * 1e3,
        "workload": f"{n_bullet_worlds} worlds x 40 fast disks and 3..8-gons (60..180 m/s, half bullets) in a "
                    f"closed 30 m box, seed 9, steps 4..{3 + bullet_steps}",
        "toi_rounds_per_step": statistics.mean(s["toiRounds"] for s in st_b),
        "toi_events_per_step": statistics.mean(s["toiContactsFound"] for s in st_b),
        "toi_computed_per_step": statistics.mean(s["toiContactsUpdatedToi"] for s in st_b),
        "cpu_baseline": {"value": res[0][1] / res[0][0], "unit": UNIT, "cores": 1, "kind": kind,
                         "sample": cpu_sample_desc(kind, n_bullet_worlds, 16, 1, 3, bullet_steps)
                         + ", time-of-impact phase on"}}
    return {"headline_batch": headline, "bullets": bullets,
            "timing": "host clock around synchronous steps (the TOI loop syncs between rounds)"}


def adjoint_bench(device, n_worlds=64, steps=240, every=16):
    """StepAdjoint on the pushing workload: 64 worlds (a disk and 32 boxes on a
    ground, seed 2), 240 steps with checkpoints every 16, loss = squared distance
    of each world's mean box centre from a target in [10,30]x[0,2].  Reports
    differentiated body-steps per second (forward with checkpoints + recorded
    recompute + reverse pass) and its cost against the plain forward steps."""
    from playrho_gb300 import gpu, scenes

    worlds = scenes.push_worlds(n_worlds, seed=2)
    rng = np.random.default_rng(2)
    targets = np.stack([rng.uniform(10, 30, n_worlds), rng.uniform(0, 2, n_worlds)], 1)
    conf = gpu.default_conf()
    n_dyn = sum(int((w.body_type == 2).sum()) for w in worlds)
    fwd = gpu.GpuBatch(worlds, device=device)
    fwd.step_n(3, conf)  # capture the graph
    fwd.close()
    fwd = gpu.GpuBatch(worlds, device=device)
    t0 = time.perf_counter()
    fwd.step_n(steps, conf)
    t_fwd = time.perf_counter() - t0
    fwd.close()
    # a warm-up window on another batch of the same worlds leaves the window's
    # device memory (checkpoints, tapes, adjoint state) cached for the timed one
    wu = gpu.GpuBatch(worlds, device=device)
    wu.adjoint_begin(every)
    wu.adjoint_forward(steps, conf)
    wu.adjoint_backward(np.zeros((wu.n_bodies, 3)), None)
    wu.adjoint_end()
    wu.close()
    g = gpu.GpuBatch(worlds, device=device)
    t0 = time.perf_counter()
    g.adjoint_begin(every)
    g.adjoint_forward(steps, conf)
    b = g.bodies()
    ybar = np.zeros((g.n_bodies, 3))
    loss = 0.0
    for k, w in enumerate(worlds):
        lo = int(g.body_base[k])
        boxes = lo + 2 + np.arange(32)  # ground, disk, then the boxes
        m = b["pos"][boxes, :2].mean(0)
        loss += float(((m - targets[k]) ** 2).sum())
        ybar[boxes, :2] = 2.0 * (m - targets[k]) / 32.0
    grads = g.adjoint_backward(ybar, None)
    t_adj = time.perf_counter() - t0
    info = g.adjoint_info()
    prof = g.adjoint_profile()
    g.adjoint_end()
    g.close()
    back_ms = prof["record_ms"] + prof["reverse_ms"]
    return {"metric": "adjoint grad body-steps/s", "value": n_dyn * steps / t_adj, "unit": "body-steps/s",
            # the gradient's own cost (recomputing each segment with its tape, then the
            # reverse pass) and the whole differentiated run (plus the checkpointed
            # forward pass that gives the loss), both over the plain forward steps
            "cost_vs_forward": back_ms / (t_fwd * 1e3), "total_vs_forward": t_adj / t_fwd,
            "forward_ms": t_fwd * 1e3, "adjoint_ms": t_adj * 1e3,
            "workload": f"{n_worlds} worlds x (disk + 32 boxes + ground), seed 2, {steps} steps, "
                        f"checkpoint every {every}, loss |mean box centre - target|^2",
            "loss": loss, "grad_norm": float(np.linalg.norm(grads["vel"])),
            "replay_mismatches": info["replay_mismatches"], "tape_overflows": info["tape_overflows"],
            "phases_ms": prof,
            "dtype": "f32 forward, f32 local derivatives", "timing": "host clock around synchronous calls"}


def adjoint_window_bench(worlds, conf, device, settle, window=64, every=8):
    """StepAdjoint over a window of the chains workload (revolute joints
    included): loss = sum over worlds of the mean x of the chains' last links,
    a window of 64 steps with checkpoints every 8.  Two batches of the same
    worlds advance in lockstep (the step is deterministic): one times the plain
    forward steps of the window, the other differentiates the same window."""
    from playrho_gb300 import gpu

    n_dyn = sum(int((w.body_type == 2).sum()) for w in worlds)
    adj = gpu.GpuBatch(worlds, device=device)
    plain = gpu.GpuBatch(worlds, device=device)
    for b in (adj, plain):
        b.step_n(settle, conf)
    # warm-up window (the plain twin steps along): leaves the window's device
    # memory cached for the timed one
    adj.adjoint_begin(every)
    adj.adjoint_forward(window, conf)
    adj.adjoint_backward(np.zeros((adj.n_bodies, 3)), None)
    adj.adjoint_end()
    plain.step_n(window, conf)
    t0 = time.perf_counter()
    plain.step_n(window, conf)
    t_fwd = time.perf_counter() - t0
    plain.close()
    # d(loss)/d(final state): the loss is linear in the tips' x, so its gradient
    # is known before the window runs (the chains' topology, not their state)
    ybar = np.zeros((adj.n_bodies, 3))
    for k, w in enumerate(worlds):
        jb = np.asarray(w.joint_bodies).reshape(-1, 2)
        tips = sorted(set(jb[:, 1].tolist()) - set(jb[:, 0].tolist()))
        ybar[int(adj.body_base[k]) + np.asarray(tips, dtype=np.int64), 0] = 1.0 / max(1, len(tips))
    t0 = time.perf_counter()
    adj.adjoint_begin(every)
    adj.adjoint_forward(window, conf)
    grads = adj.adjoint_backward(ybar, None)
    t_adj = time.perf_counter() - t0
    info = adj.adjoint_info()
    prof = adj.adjoint_profile()
    adj.adjoint_end()
    adj.adjoint_trim()
    adj.close()
    back_ms = prof["record_ms"] + prof["reverse_ms"]
    return {"metric": "adjoint grad body-steps/s", "value": n_dyn * window / t_adj, "unit": "body-steps/s",
            "cost_vs_forward": back_ms / (t_fwd * 1e3), "total_vs_forward": t_adj / t_fwd,
            "forward_ms": t_fwd * 1e3, "adjoint_ms": t_adj * 1e3,
            "workload": f"{len(worlds)} chain worlds (revolute joints) after {settle + window} steps, window "
                        f"{window} steps, checkpoint every {every}, loss = mean x of the chains' last links",
            "grad_norm": float(np.linalg.norm(grads["vel"])),
            "replay_mismatches": info["replay_mismatches"], "tape_overflows": info["tape_overflows"],
            "phases_ms": prof, "dtype": "f32 forward, f32 local derivatives",
            "timing": "host clock around synchronous calls"}


def nvtx_ranges():
    """(push, pop) of an NVTX range, or no-ops without torch's NVTX binding."""
    try:
        import torch

        return torch.cuda.nvtx.range_push, torch.cuda.nvtx.range_pop
    except Exception:
        return (lambda name: None), (lambda: None)


def launches_per_step(batch) -> int:
    """Kernel nodes in the captured step graph (counted from the graph itself)."""
    import ctypes

    n = ctypes.c_uint32()
    rc = batch.lib.prgpu_graph_kernel_count(batch.h, ctypes.byref(n))
    return int(n.value) if rc == 0 else -1


def main():
    args = parse()
    rank, world_size, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world_size, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
