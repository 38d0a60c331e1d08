#!/usr/bin/env python3
"""Benchmark of the GB300 EC-FDTD engine (prints one JSON line on rank 0).

A "step" is one full EC-FDTD timestep (voltage + current half-steps with every extension and
the per-step probe processing) over the whole mesh of the workload.  Default workload: the
bandwidth-stress configuration, 512x512x256 mesh lines (67.1 M cells, 1.9 GB of field state,
larger than the 129 MB L2), seeded random dielectric / lossy / Drude-Lorentz blocks, Mur walls,
4 Gaussian point sources with per-step voltage monitors.

value   = cells * K / device time of K steps replayed through the captured step graph (MCells/s)
e2e     = the same metric through the C ABI with host buffers: per step one oems_cuda_iterate(1)
          plus a device->host read of every probe's newest sample (the openEMS processing loop)
roofline= algorithmic bytes of the dominant kernel (36 B per cell per half-step update: read the
          updated field, read the other field, write the updated field) over its average
          CUDA-event duration, against the measured HBM copy bandwidth
cpu_baseline = openEMS's multithreaded SSE-compressed engine on the host cores (all cores) on a
          bounded number of steps of the same workload: the reference's own engine compiled from
          its sources (oracle/_ref) where that build exists on the host, else the C restatement
          of it (oracle port); ``kind`` says which.  cpu_thread_sweep repeats it at 1, 2, 4, ...
          threads.
configs = the 100^3 vacuum cube and the 160x160x80 patch (UPML, lumped port, NF2FF boxes) on the
          GPU: both largely L2-resident, so they report MCells/s only
e2e_job = the whole stress job as a user runs it: operator build, engine setup, the
          configuration's 2000 steps with every probe sample read back, teardown

Multi-GPU: replicas only (one independent simulation per rank, no collective on the data path);
``value`` is the sum over ranks.
"""
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

ALG_BYTES_PER_CELL_STEP = 72          # V: r/w 12+12, I read 12; I: r/w 12+12, V read 12
ALG_BYTES_PER_CELL_HALF = 36


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_from_profiles(kernel):
    """Per-cell DRAM bytes of a kernel from the committed ncu summary (None if absent)."""
    path = os.path.join(ROOT, "profiles", "ncu_update_kernels_stress.md")
    try:
        for line in open(path):
            if line.startswith(f"traffic_bytes_per_cell[{kernel}]"):
                return float(line.split("=")[1].split()[0])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.file:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def build_workload(name, shape=None):
    from openems_gb300 import configs
    if name == "stress":
        shape = tuple(shape) if shape else (512, 512, 256)
        return (configs.stress(shape=shape, steps=100000),
                "stress %dx%dx%d lines, 64 random blocks (10%% Drude/Lorentz), Mur x6, 4 sources" % shape)
    if name == "stress_upml":
        shape = tuple(shape) if shape else (512, 512, 256)
        return (configs.stress(shape=shape, steps=100000, bc=(3,) * 6, dispersive=False),
                "stress %dx%dx%d lines, 64 random blocks, UPML 8 x6, 4 sources" % shape)
    if name == "patch":
        return configs.patch(steps=100000), "patch 160x160x80 graded, UPML 8, 50 Ohm port, NF2FF 3 freqs"
    if name == "plain":
        n = int(shape[0]) if shape else 100
        return configs.plain_cube(n=n, steps=100000), "plain %d^3, vacuum, PEC, soft Ez, V/I probes" % n
    if name == "design":
        case = configs.DesignCase(steps=100000)
        return (case.build(case.eps0)[1],
                "design 200x200x100 lines, 0.5 mm, UPML 8, 64x64x16 eps_r cells, two 50 Ohm ports")
    raise SystemExit(f"unknown workload {name}")


def cpu_engine(op, max_ts, threads):
    """The CPU engine timed as the reference: openEMS's own multithreaded engine compiled from
    its sources (oracle/_ref) where it was built on this host, else the C restatement of it
    (the oracle port; the reference sources are not on every host).  Returns (engine, kind)."""
    try:
        from oracle import refengine
        if refengine.available():
            return refengine.RefEngine(op, max_ts, kind="multithread", threads=threads), "reference"
    except Exception:
        pass
    from oracle.oracle import OracleEngine
    return OracleEngine(op, max_ts, threads=threads), "port"


def cpu_baseline(op, steps_cap, budget_s, threads, engine=None):
    """openEMS's multithreaded SSE-compressed engine on the host cores, stepping like its
    processing loop (one step, then the probes)."""
    if engine is None:
        eng, kind = cpu_engine(op, steps_cap + 2, threads)
    else:
        eng, kind = engine
    eng.IterateTS(1)                        # warm-up step (threads started, pages touched)
    n = 0
    t0 = time.perf_counter()
    while n < steps_cap:
        eng.IterateTS(1)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    eng.close()
    cells = float(np.prod(op.num_lines.astype(np.float64)))
    return cells * n / dt / 1e6, n, dt, kind


def cpu_thread_sweep(op, budget_s, nproc):
    """The CPU engine at 1, 2, 4, ... threads up to nproc (a bounded sample of steps each)."""
    out = {}
    t = 1
    counts = []
    while t < nproc:
        counts.append(t)
        t *= 2
    counts.append(nproc)
    for t in counts:
        v, n, sec, kind = cpu_baseline(op, 50, budget_s, t)
        out[str(t)] = {"mcells_s": round(v, 1), "steps": n, "seconds": round(sec, 2), "kind": kind}
    return out


def processing_loop(eng, steps, slot):
    """openEMS's processing loop through the C ABI: per step oems_cuda_iterate(1), then a read of
    every probe's newest sample.  Python's cyclic garbage collector is paused for the loop (it
    allocates only the small result arrays): a collection sweeping the objects the earlier
    measurements left behind would otherwise land in the timing.  Returns the wall seconds."""
    import gc
    pids = eng.vprobe_ids + eng.iprobe_ids
    was = gc.isenabled()
    gc.disable()
    try:
        t0 = time.perf_counter()
        for _ in range(steps):
            eng.IterateTS(1)
            slot += 1
            for pid in pids:
                eng.probe_range(pid, slot, 1)
        return time.perf_counter() - t0
    finally:
        if was:
            gc.enable()


def measure_config(name, steps, e2e_steps=200, cpu_budget=0.0):
    """One more configuration on the GPU: device-timed MCells/s over `steps` replayed steps, and
    MCells/s end to end through the C ABI (iterate(1) + a synchronous read of every probe's new
    sample per step, openEMS's processing loop); with cpu_budget > 0 also the CPU engine on every
    host core for about that many seconds of steps."""
    from openems_gb300.engine import Engine_CUDA
    from openems_gb300.operator import build_device
    t0 = time.perf_counter()
    with build_device("cuda" if name != "design" else "cpu"):
        op, desc = build_workload(name)
    t_build = time.perf_counter() - t0
    cells = float(np.prod(op.num_lines.astype(np.float64)))
    eng = Engine_CUDA(op, steps + e2e_steps + 96)
    eng.IterateTS(80)               # warm-up; also where the engine picks its step form (>= 4 graphs)
    eng.sync()
    ms = eng.timed_iterate(steps)
    e2e_s = processing_loop(eng, e2e_steps, eng.GetNumberOfTimesteps())
    state_mb = 24 * cells / 1e6
    out = {"workload": desc, "cells": cells, "steps": steps, "mcells_s": cells * steps / (ms / 1e3) / 1e6,
           "ms_per_step": ms / steps, "e2e_mcells_s": cells * e2e_steps / e2e_s / 1e6, "e2e_steps": e2e_steps,
           "build_s": round(t_build, 2), "launches_per_step": eng.launches_per_step(),
           "l2": "field state %.0f MB against a 129 MB L2: largely L2-resident, so no HBM fraction is claimed"
                 % state_mb}
    eng.close()
    if cpu_budget > 0:
        nproc = os.cpu_count() or 1
        v, n, sec, kind = cpu_baseline(op, 100000, cpu_budget, nproc)
        out["cpu"] = {"mcells_s": round(v, 1), "steps": n, "seconds": round(sec, 2), "cores": nproc, "kind": kind}
    return out


def measure_batched(count):
    """Batched form: `count` seeded instances (lines U[48,160]^3, 0.5-2 mm, UPML 8, dielectric
    block, 50 Ohm port, steps U[4000,12000]) run serially (one engine after the other, each
    replaying its step graph) and then together (persistent launches in one graph); sims/s of
    both, wall clock around the run calls with the device synchronised, setup excluded."""
    from openems_gb300 import configs
    from openems_gb300.batch import BatchEngine
    from openems_gb300.engine import Engine_CUDA
    t0 = time.perf_counter()
    inst = [configs.batch_instance(1000 + k) for k in range(count)]
    t_build = time.perf_counter() - t0
    steps = [s for _, s in inst]
    cells = [float(np.prod(op.num_lines.astype(np.float64))) for op, _ in inst]
    cell_steps = sum(c * s for c, s in zip(cells, steps))
    # serial: one engine at a time
    serial_s = 0.0
    per_inst = []
    for op, s in inst:
        e = Engine_CUDA(op, s)
        e.sync()
        t = time.perf_counter()
        e.IterateTS(s)
        e.sync()
        dt = time.perf_counter() - t
        serial_s += dt
        per_inst.append([int(np.prod(op.num_lines.astype(np.float64))), s, round(dt, 4)])
        e.close()
    # serial in openEMS's processing-loop style (RunFDTD, openems.cpp:1427-1431): with probes
    # sampled every step the loop runs IterateTS(1) and then reads the probes on the host
    loop_s = 0.0
    for op, s in inst:
        e = Engine_CUDA(op, s)
        e.sync()
        loop_s += processing_loop(e, s, 0)
        e.close()
    engines = [Engine_CUDA(op, s) for op, s in inst]
    for e in engines:
        e.sync()
    be = BatchEngine(engines)
    t = time.perf_counter()
    be.run(steps)
    batch_s = time.perf_counter() - t
    cfg = be.config()
    # every instance's port V/I series against a serial rerun of two instances (spot check)
    same = True
    for k in (0, count - 1):
        e = Engine_CUDA(inst[k][0], steps[k])
        e.IterateTS(steps[k])
        for pid in e.vprobe_ids + e.iprobe_ids:
            same &= bool(np.array_equal(e.probe_series(pid), engines[k].probe_series(pid), equal_nan=True))
        e.close()
    be.close()
    for e in engines:
        e.close()
    return {"instances": count, "sims_per_s_batched": count / batch_s, "sims_per_s_serial": count / serial_s,
            "speedup": serial_s / batch_s, "batched_s": batch_s, "serial_s": serial_s,
            "sims_per_s_serial_processing_loop": count / loop_s, "speedup_vs_processing_loop": loop_s / batch_s,
            "serial_processing_loop_s": loop_s,
            "mcells_per_s_batched": cell_steps / batch_s / 1e6, "mcells_per_s_serial": cell_steps / serial_s / 1e6,
            "total_cells": sum(cells), "steps_min_max": [min(steps), max(steps)], "tuned": cfg,
            "series_equal_serial_spot_check": same, "build_s": round(t_build, 1),
            "serial_per_instance_cells_steps_s": per_inst}


def batch_launch_case(count=32, steps=40):
    """The batched-form instances for an ncu launch list: the largest instance alone for 48 steps
    (its own split kernels from its graphs), then all `count` together for `steps` steps in
    per-phase launches (one launch per phase over every instance)."""
    from openems_gb300 import configs
    from openems_gb300.batch import BatchEngine
    from openems_gb300.engine import Engine_CUDA
    inst = [configs.batch_instance(1000 + k) for k in range(count)]
    big = max(range(count), key=lambda k: np.prod(inst[k][0].num_lines))
    e = Engine_CUDA(inst[big][0], 64)
    e.IterateTS(48)
    e.sync()
    kernels = e.update_kernels()
    e.close()
    engines = [Engine_CUDA(op, steps + 8) for op, _ in inst]
    be = BatchEngine(engines)
    be.run([steps] * count, block_size=256, depth=1 | 0x80000000)
    cfg = be.config()
    be.close()
    for x in engines:
        x.close()
    return {"serial_instance": int(big), "lines": inst[big][0].num_lines.tolist(), "kernels": kernels, "batch": cfg}


def measure_adjoint(steps=8000):
    """Differentiable form: 200x200x100 lines at 0.5 mm, UPML 8, 64x64x16 design cells of eps_r
    U[1,6] (seeded), 50 Ohm input and output ports 60 cells from the region, objective = port
    power at 4/5/6 GHz over 8000 steps, checkpoints every 256 steps.  Device times (CUDA events
    on the engine stream): a plain forward run (step graph replay), the checkpointed forward run
    and the reverse sweep (recompute + adjoint kernels)."""
    from openems_gb300.adjoint import AdjointRun
    from openems_gb300.configs import DesignCase
    from openems_gb300.engine import Engine_CUDA
    t0 = time.perf_counter()
    case = DesignCase(steps=steps)
    _, data = case.build(case.eps0)
    t_build = time.perf_counter() - t0
    eng = Engine_CUDA(data, case.steps)
    plain_ms = eng.timed_iterate(case.steps)
    eng.close()
    out = {"config": "200x200x100 lines, 0.5 mm, UPML 8, design 64x64x16, %d steps" % steps,
           "forward_ms": plain_ms, "build_s": round(t_build, 1)}
    cells = float(np.prod(data.num_lines.astype(np.float64)))
    out["forward_mcells_per_s"] = cells * case.steps / plain_ms / 1e3
    for K, tag in ((256, "checkpoint_256"), (0, "record")):
        run = AdjointRun(case, case.eps0, checkpoint_every=K)
        try:
            g_eps, g_kap = run.gradient()
            tm = run.timing()
            J = run.J
        finally:
            run.close()
        # the objective is a port power in SI units (about 1e-40 W here); the normalised forms
        # show the gradients are well resolved in double: d(ln J)/d(eps_r) and d(ln J)/d(kappa)
        out[tag] = {"forward_ms": tm["forward_ms"], "backward_ms": tm["backward_ms"],
                    "adjoint_over_forward": tm["backward_ms"] / plain_ms,
                    "gradient_over_forward": (tm["forward_ms"] + tm["backward_ms"]) / plain_ms,
                    "launches_per_reverse_step": tm["launches_per_reverse_step"],
                    "objective": J, "grad_eps_norm": float(np.linalg.norm(g_eps)),
                    "grad_kappa_norm": float(np.linalg.norm(g_kap)),
                    "dlnJ_deps_norm": float(np.linalg.norm(g_eps) / abs(J)) if J else None,
                    "dlnJ_dkappa_norm": float(np.linalg.norm(g_kap) / abs(J)) if J else None,
                    "dlnJ_deps_max": float(np.max(np.abs(g_eps)) / abs(J)) if J else None}
    return out


def measure_nf2ff(steps=2000, cpu_angles=64):
    """NF2FF far-field transform of the patch workload's NF2FF box (160x160x80 graded lines, six
    faces, E and H FD dumps at 1.5/2/2.5 GHz) after `steps` timesteps: the device transform over
    the full sphere at 1 degree (181 x 361 angles) per frequency (wall clock around the call,
    which synchronises), and the numpy restatement on the host cores for `cpu_angles` angles,
    scaled per angle."""
    from openems_gb300 import configs
    from openems_gb300.engine import Engine_CUDA
    from openems_gb300.nf2ff import box_faces, calc_nf2ff
    from oracle.nf2ff_ref import nf2ff as nf2ff_host
    op = configs.patch(steps=steps)
    eng = Engine_CUDA(op, steps)
    eng.IterateTS(steps)
    faces = box_faces(eng)
    samples = sum(int(np.prod([len(c) for c in f[2]])) for f in faces)
    theta = np.deg2rad(np.arange(0, 181, 1.0))
    phi = np.deg2rad(np.arange(0, 361, 1.0))
    calc_nf2ff(eng, 0, theta[:8], phi[:8])                   # warm-up
    t0 = time.perf_counter()
    res = [calc_nf2ff(eng, fi, theta, phi) for fi in range(3)]
    gpu_s = (time.perf_counter() - t0) / 3
    data = [(c, eng.fd_dump(ie)[0], eng.fd_dump(ih)[0]) for ie, ih, c in faces]
    th_s = np.deg2rad(np.linspace(0, 180, cpu_angles))
    t0 = time.perf_counter()
    nf2ff_host(data, res[0].freq, th_s, phi[:1])
    cpu_s = time.perf_counter() - t0
    eng.close()
    nang = len(theta) * len(phi)
    return {"config": "patch 160x160x80, NF2FF box of 6 faces, 1 deg sphere (181x361), per frequency",
            "face_samples": samples, "angles": nang, "gpu_ms_per_freq": gpu_s * 1e3,
            "sample_angle_pairs_per_s": samples * nang / gpu_s,
            "cpu_oracle_ms_per_freq_scaled": cpu_s / cpu_angles * nang * 1e3,
            "cpu_sample": f"{cpu_angles} angles, numpy restatement (oracle/nf2ff_ref.py)",
            "Dmax": [r.Dmax for r in res], "Prad_W": [r.Prad for r in res]}


def max_over_ranks(value, dist=None, device="cuda"):
    """The slowest rank's value, on every rank (the timed region is bracketed by barriers)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mcells(cells, steps, ms, world):
    """MCells/s of all ranks together: each rank runs its own replica of `cells` cells."""
    return cells * steps / (ms / 1e3) / 1e6 * world


def run_reference(args, op, desc, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    cells = float(np.prod(op.num_lines.astype(np.float64)))
    eng, kind = cpu_engine(op, args.steps + args.warmup + 2, threads)
    eng.IterateTS(max(args.warmup, 1))
    t0 = time.perf_counter()
    done = 0
    budget = float(os.environ.get("OEMS_REF_BUDGET_S", "120"))
    while done < args.steps:
        eng.IterateTS(1)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    eng.close()
    v = cells * done / dt / 1e6
    line = {
        "impl": "reference", "metric": "MCells/s", "value": v, "unit": "MCells/s", "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": dt / done * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "cells": cells},
        "cpu_baseline": {"value": v, "unit": "MCells/s", "cores": threads, "kind": kind,
                         "sample": f"{done} timesteps of the full workload (bounded to {budget:.0f} s), "
                                   "one step then the probes, as openEMS's processing loop runs"},
        "e2e": {"value": v, "unit": "MCells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="stress", choices=["stress", "stress_upml", "patch", "plain", "design"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--shape", default=None, help="mesh lines of the stress workload, e.g. 256,256,192")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-form measurement")
    ap.add_argument("--batch-count", type=int, default=32)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-form measurement")
    ap.add_argument("--no-nf2ff", action="store_true", help="skip the NF2FF far-field measurement")
    ap.add_argument("--adjoint-steps", type=int, default=8000,
                    help="timesteps of the differentiable-form measurement (8000 = its configuration)")
    ap.add_argument("--no-configs", action="store_true", help="skip the 100^3 cube and patch measurements")
    ap.add_argument("--no-cpu-sweep", action="store_true", help="skip the CPU thread sweep")
    ap.add_argument("--sweep-budget", type=float, default=3.0, help="seconds per thread count of the CPU sweep")
    ap.add_argument("--job-steps", type=int, default=2000,
                    help="steps of the whole-job measurement (2000 = the stress configuration's)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference" and rank != 0:
        return
    shape = [int(v) for v in args.shape.split(",")] if args.shape else None
    if args.impl == "reference":
        op, desc = build_workload(args.workload, shape)
        run_reference(args, op, desc, rank)
        return
    # operator setup: the per-edge numerics on the GPU (bit-identical to the host build) where
    # the geometry allows it; the host build is timed beside it once
    from openems_gb300.operator import build_device
    dev = "cpu" if args.workload == "design" else "cuda"
    t_build = time.perf_counter()
    with build_device(dev):
        op, desc = build_workload(args.workload, shape)
    t_build = time.perf_counter() - t_build
    t_build_host = None

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    from openems_gb300.engine import Engine_CUDA
    cells = float(np.prod(op.num_lines.astype(np.float64)))
    e2e_steps = min(args.steps, 100)
    prof_steps = min(args.steps, 20)
    total = args.warmup + args.steps + prof_steps + e2e_steps + 4
    t_setup = time.perf_counter()
    eng = Engine_CUDA(op, total, device=local if world > 1 else 0)
    t_setup = time.perf_counter() - t_setup
    eng.IterateTS(max(args.warmup, 3))
    eng.sync()

    # ---- timed region: K steps through the captured graph -------------------------------
    if dist:
        dist.barrier()
    eng.sync()
    with ClockSampler(local) as clk:
        ms = eng.timed_iterate(args.steps)
    clocks = clk.summary()
    ms = max_over_ranks(ms, dist, "cuda") if dist else ms
    value = whole_job_mcells(cells, args.steps, ms, world)

    # ---- per-kernel event timing for the roofline ----------------------------------------
    from openems_gb300._native import KERNEL_CLASSES
    kms, kcnt = eng.profile(prof_steps)
    kernels = {KERNEL_CLASSES[i]: {"ms_total": kms[i], "launches": kcnt[i]} for i in range(len(KERNEL_CLASSES)) if kcnt[i]}
    dom = max(("update_v", "update_i"), key=lambda k: kms[KERNEL_CLASSES.index(k)])
    di = KERNEL_CLASSES.index(dom)
    avg_ms = kms[di] / max(kcnt[di], 1)
    achieved = ALG_BYTES_PER_CELL_HALF * cells / (avg_ms / 1e3) / 1e9
    peak, peak_kind = _peaks()
    tr = _traffic_from_profiles(dom) if args.workload == "stress" else None   # measured for that mesh
    kname = eng.update_kernels()[0 if dom == "update_v" else 1]
    alg_launch = ALG_BYTES_PER_CELL_HALF * cells
    if kname == "k_step_march":
        # one kernel per step (the per-kernel profile times the separate kernels): the step's 72 B
        # per cell over the replayed step time; the march itself moves about 52 B per cell
        achieved = ALG_BYTES_PER_CELL_STEP * cells / (ms / args.steps / 1e3) / 1e9
        alg_launch = ALG_BYTES_PER_CELL_STEP * cells
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": tr * cells if tr is not None else None,
                "alg_bytes_per_launch": alg_launch,
                "step_frac": (ALG_BYTES_PER_CELL_STEP * cells / (ms / args.steps / 1e3) / 1e9) / peak}

    # ---- end to end through the C ABI: iterate(1) + D2H of the newest probe samples -------
    pids = eng.vprobe_ids + eng.iprobe_ids
    e2e_s = processing_loop(eng, e2e_steps, eng.GetNumberOfTimesteps())
    e2e = {"value": cells * e2e_steps / e2e_s / 1e6 * world, "unit": "MCells/s", "h2d_bytes_per_step": 0,
           "d2h_bytes_per_step": 8 * len(pids), "steps": e2e_steps,
           "note": "per step: oems_cuda_iterate(1) then oems_cuda_read_probe_range of every probe (synchronous)"}
    launches = eng.launches_per_step()
    eng.close()

    # ---- the whole job as a user runs it: operator build, engine setup, the configuration's
    # steps in openEMS's processing style (probe samples read back every step), teardown --------
    e2e_job = None
    if rank == 0 and args.workload == "stress" and args.job_steps > 0:
        t0 = time.perf_counter()
        with build_device(dev):
            jop, _ = build_workload(args.workload, shape)
        t1 = time.perf_counter()
        jeng = Engine_CUDA(jop, args.job_steps + 2)
        t2 = time.perf_counter()
        processing_loop(jeng, args.job_steps, 0)
        t3 = time.perf_counter()
        jeng.close()
        t4 = time.perf_counter()
        e2e_job = {"value": cells * args.job_steps / (t4 - t0) / 1e6, "unit": "MCells/s",
                   "steps": args.job_steps, "seconds": round(t4 - t0, 3), "build_s": round(t1 - t0, 3),
                   "engine_setup_s": round(t2 - t1, 3), "steps_s": round(t3 - t2, 3),
                   "teardown_s": round(t4 - t3, 3),
                   "note": "operator build + engine setup + every step with its probe samples read back + teardown"}

    batched = None
    if rank == 0 and not args.no_batch:
        batched = measure_batched(args.batch_count)

    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = measure_adjoint(args.adjoint_steps)

    nf2ff = None
    if rank == 0 and not args.no_nf2ff:
        nf2ff = measure_nf2ff()

    others = None
    if rank == 0 and not args.no_configs:
        cb = 0.0 if args.no_cpu_baseline else 3.0
        others = {"plain_100": measure_config("plain", 2000, cpu_budget=cb),
                  "patch_160x160x80": measure_config("patch", 1000, cpu_budget=cb)}

    base = None
    sweep = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, n, sec, kind = cpu_baseline(op, 50, args.cpu_budget, threads)
        base = {"value": v, "unit": "MCells/s", "cores": threads, "kind": kind,
                "sample": f"{n} timesteps of the full {desc} workload ({sec:.1f} s, setup excluded)"}
        if not args.no_cpu_sweep:
            sweep = cpu_thread_sweep(op, args.sweep_budget, threads)

    # the host build for comparison, last: its several GB of temporary arrays would otherwise
    # disturb the allocations of the whole-job measurement above
    if rank == 0 and dev == "cuda" and not args.no_cpu_baseline:
        t0 = time.perf_counter()
        build_workload(args.workload, shape)
        t_build_host = time.perf_counter() - t0

    if rank == 0:
        line = {
            "metric": "MCells/s", "value": value, "unit": "MCells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "cells": cells, "l2": "inputs larger than L2 (field state %.2f GB)" % (
                24 * cells / 1e9), "parallelism": "replicas" if world > 1 else "single",
                "operator_classes": None, "build_s": round(t_build, 2), "build_device": dev,
                "host_build_s": round(t_build_host, 2) if t_build_host is not None else None,
                "engine_setup_s": round(t_setup, 1)},
            "roofline": roofline,
            "cpu_baseline": base,
            "cpu_thread_sweep": sweep,
            "e2e": e2e,
            "e2e_job": e2e_job,
            "configs": others,
            "clocks": clocks,
            "gpu_launches": launches * args.steps,
            "launches_per_step": launches,
            "kernels": kernels,
            "batched": batched,
            "adjoint": adjoint,
            "nf2ff": nf2ff,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
