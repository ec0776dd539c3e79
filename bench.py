#!/usr/bin/env python3
"""Benchmark: RPY mobility apply, pair-interactions/sec, on GB300.

Workload (the RPY apply microbenchmark): N blobs of radius a = 1 placed
uniformly in a cube sized for volume fraction 0.05, rejection below
separation 2.2a; forces and torques i.i.d. N(0,1) per component; the 6-dof
segment formula (Mss_mult, cuda_functions.cu:246-425) over all N x N pairs,
self pair included.  One step = one full apply.  Default N = 131072.

  value      pair-interactions/s with inputs resident in HBM (C-ABI call on
             device arrays: gmi_Mss_mult), FP32C precision by default
  e2e        the same metric through gmi_Mss_mult with host buffers: the
             pinned host->device copy of X and F and the device->host copy of
             V are inside every timed step
  roofline   compute bound on the FP32 (or FP64) FMA pipe: algorithmic FLOPs
             (87 per pair) / apply time, against the pipe peak measured on
             this GPU by gmi_measure_fma_peak
  cpu_baseline the FP64 CPU oracle (rpy_oracle.c) on a bounded target slice,
             all host cores
  time_steps time-steps/sec of the whole implicit time step (gmi_sim_step:
             Broyden, GMRES, every pair sum) on seeded free swimmers
             (1 sphere of 642 blobs with 16 x 20 segments; 1 sphere of 4096
             blobs with 640 x 20 segments), plain FP64 against FP32C pair
             sums with FP64 solves, with the velocity error between the two;
             and (config4) the aggregate rate of 64 independent swimmers of
             uneven size, one stream and host thread each, with the
             per-swimmer error

Runs one replica per GPU under torchrun (the apply does not shard here:
"replicas only"), max-over-ranks time, rank 0 prints one JSON line.
``--impl reference`` times the reference algorithm's CPU restatement instead.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOP_PER_PAIR_SS = 87  # canonical algorithmic FLOPs per segment-segment pair (FMA = 2)
# DRAM bytes (read + write) of one launch of the apply's pair kernel, from an
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum, one pass) of this
# benchmark with the shape pinned: (n, precision, threads, targets, splits,
# sources per step) -> bytes.  Beyond the records (48 B per particle read) and
# V (48 B written), the traffic is the FP64 split partial sums.
PAIR_KERNEL_TRAFFIC = {(131072, "fp32c", 256, 1, 8, 2): 7976192, (131072, "fp32c", 64, 1, 4, 2): 7011584,
                       (131072, "fp32c", 64, 1, 8, 2): 8071168}
METRIC = "RPY pair-interactions/sec"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gmi", "reference"], default="gmi")
    p.add_argument("--n", "--particles", dest="n", type=int, default=131072,
                   help="particles of the apply benchmark (--particles under torchrun, whose parser takes --n*)")
    p.add_argument("--precision", choices=["fp32c", "fp64"], default="fp32c")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 side measurement")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU sample")
    p.add_argument("--no-autotune", action="store_true", help="use the default launch shape (profiling)")
    p.add_argument("--shape", default=None,
                   help="pin the apply's launch shape instead of autotuning: threads,targets,splits,sources_per_step "
                        "(the traffic capture pins the shape the autotuner picks)")
    p.add_argument("--ts-workloads", default="config1,config3,config4,config1_beat,config3_beat,config5",
                   help="time-step workloads (comma separated; empty to skip)")
    p.add_argument("--ts-steps", default="config1:100,config3:10,config4:2,config1_beat:100,config3_beat:100,"
                                         "config5:1", help="timed steps per workload")
    p.add_argument("--ts-warmup", type=int, default=5, help="untimed steps before the timed ones")
    p.add_argument("--ts-warmups", default="config4:1,config5:1",
                   help="untimed steps per workload where they differ from --ts-warmup")
    p.add_argument("--ts-fp32c-only", default="config5",
                   help="workloads whose plain FP64 run is skipped (config 5's FP64 steps take minutes each; "
                        "pass an empty value to measure them)")
    p.add_argument("--accuracy-swimmers", type=int, default=8,
                   help="swimmers of the config-4 accuracy check against a tight-tolerance FP64 run (0 to skip)")
    p.add_argument("--learned", default="config3",
                   help="workloads of the learned initial inverse Jacobian A/B (comma separated; empty to skip)")
    p.add_argument("--learned-data-steps", type=int, default=15,
                   help="plain time steps of the training geometry whose secant pairs train the network")
    p.add_argument("--learned-train-steps", type=int, default=2000, help="Adam steps of the network")
    p.add_argument("--ts-swimmers", type=int, default=64, help="swimmers of a batch time-step workload (config4)")
    return p.parse_args()


# --------------------------------------------------------------------------
# distributed plumbing (replicas only; the collective is for timing)
# --------------------------------------------------------------------------
def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# --------------------------------------------------------------------------
# workload
# --------------------------------------------------------------------------
def make_inputs(n: int, seed: int = 2026):
    from generic_mobility_interface_class_gb300 import seeding
    x = seeding.random_cube(n, min_sep=2.2, phi=0.05, a=1.0, seed=seed)
    f = np.random.default_rng(seed + 1).normal(size=(n, 6))
    return x, f


def cpu_sample(x, f, seconds: float, keep: bool = False):
    """FP64 CPU oracle on the target slice [0, nt) sized for ~`seconds` of
    work.  Returns (nt, seconds taken, cores, the slice's velocities when
    keep is set)."""
    from oracle import rpy
    n = x.shape[0]
    probe = min(n, 256)
    t0 = time.perf_counter()
    rpy.mss(x, f, targets=(0, probe))
    dt = max(time.perf_counter() - t0, 1e-6)
    nt = int(min(n, max(probe, probe * seconds / dt)))
    t0 = time.perf_counter()
    v = rpy.mss(x, f, targets=(0, nt))
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return nt, dt, cores, (v if keep else None)


def per_target_error(got, want):
    """Max and RMS over targets of |got_i - want_i| / |want_i|, for the
    velocity and the angular velocity of each target separately, and the
    max-normalised error max|got - want| / max|want|."""
    g = np.asarray(got, dtype=np.float64).reshape(-1, 3)
    w = np.asarray(want, dtype=np.float64).reshape(-1, 3)
    r = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)
    return {"max_rel_per_target": float(r.max()), "rms_rel_per_target": float(np.sqrt(np.mean(r * r))),
            "max_normalised": float(np.abs(g - w).max() / np.abs(w).max())}


def run_reference(args, world, rank):
    """Reference arm: the reference algorithm on the host cores (the oracle
    port of cuda_functions.cu's Mss_mult; the reference's own host build
    cannot run on this host), bounded target slice per step.  Beside it
    (``cuda_on_gb300``), the reference's own CUDA kernel built for sm_103a,
    timed on the GPU, where its build is present."""
    if rank != 0:
        return
    from oracle import rpy
    rpy.build(with_reference=False)
    x, f = make_inputs(args.n)
    n = x.shape[0]
    nt, dt, cores, _ = cpu_sample(x, f, max(1.0, min(args.cpu_seconds, 60.0) / max(args.steps, 1)))
    for _ in range(args.warmup):
        rpy.mss(x, f, targets=(0, min(nt, 64)))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rpy.mss(x, f, targets=(0, nt))
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = nt * n * args.steps / total
    cuda = reference_cuda_timing(x, f, nt)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"RPY apply microbenchmark, N={n} (cube, phi=0.05, min sep 2.2a, 6-dof Mss)",
                   "n": n, "sample_targets": nt, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": f"{nt} targets x {n} sources per step"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if cuda is not None:
        line["cuda_on_gb300"] = cuda
    print(json.dumps(line), flush=True)


def reference_cuda_timing(x, f, nt, launches: int = 2):
    """The reference's own Mss_mult (cuda_functions.cu:246-425) built for
    sm_103a with this N compiled in (oracle/ref_gpu.py), launched as its
    solver launches it (64 threads per block), timed with CUDA events on
    device-resident inputs; its result on targets [0, nt) against the FP64
    CPU oracle.  None without a GPU or without the build."""
    try:
        import torch
        from oracle import ref_gpu, rpy
        n = x.shape[0]
        if not (torch.cuda.is_available() and ref_gpu.available(n)):
            return None
        k = ref_gpu.RefKernels(n)
        X = torch.as_tensor(x, device="cuda")
        F = torch.as_tensor(f, device="cuda")
        V = torch.empty((n, 6), dtype=torch.float64, device="cuda")
        k.mss(V, F, X)  # warm-up
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(launches):
            k.mss(V, F, X)
        b.record(stream)
        torch.cuda.synchronize()
        sec = a.elapsed_time(b) / 1e3 / launches
        got = V[:nt].cpu().numpy()
        k.close()
        want = rpy.mss(x, f, targets=(0, nt))
        return {"value": float(n) * n / sec, "unit": "pairs/s", "ms_per_launch": 1e3 * sec, "launches": launches,
                "dtype": "f64", "build": "reference cuda_functions.cu, nvcc -gencode arch=compute_103a,code=sm_103a "
                                         "-O3, sizes compiled in, 64 threads per block",
                "error_vs_cpu_oracle": per_target_error(got, want)}
    except Exception as e:  # the CPU arm stands without it
        return {"error": f"{type(e).__name__}: {e}"}


final_fp64 = {}  # the FP64 runs' final state per workload: the yardstick of the learned A/B


def run_learned_ab(args, dev):
    """The learned initial inverse Jacobian against the plain start, FP32C
    pair sums with FP64 solves, on the time-step workloads: the network is
    trained on the secant pairs of a plain run of the same workload built
    from another seed (another geometry), then both starts run the
    benchmark geometry from the same initial state (the policy's
    calibration steps fall in the warm-up).  Reports Broyden and GMRES
    counts, time-steps/sec, the policy's final state, and each run's
    swimmer-velocity error against the FP64 run of the same steps."""
    import torch
    from generic_mobility_interface_class_gb300 import learned, workloads
    from generic_mobility_interface_class_gb300.sim import Simulation
    from generic_mobility_interface_class_gb300._lib import GMI_FP32C
    warm_for = dict(kv.split(":") for kv in getattr(args, "ts_warmups", "").split(",") if kv)
    steps_for = dict(kv.split(":") for kv in args.ts_steps.split(",") if kv)
    out = {}
    for name in [w for w in args.learned.split(",") if w]:
        desc, make = workloads.WORKLOADS[name]
        t0 = time.perf_counter()
        records = learned.collect_secant_pairs(make(seed=2027), steps=args.learned_data_steps, capacity=50000,
                                               device=dev)
        collect_s = time.perf_counter() - t0
        net = learned.LearnedJacobian(nseg=20, device=dev)
        loss0 = net.loss(records)
        t0 = time.perf_counter()
        losses = net.train(records, steps=args.learned_train_steps, batch=512, lr=1e-3)
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0
        loss1 = net.loss(records)
        kw = make()
        warm = int(warm_for.get(name, args.ts_warmup))
        nsteps = int(steps_for.get(name, 10))
        runs = {}
        for label in ("plain", "learned"):
            sim = Simulation(**kw, precision=GMI_FP32C, device=dev)
            sim.prepare()
            if label == "learned":
                sim.set_learned_jacobian(net, learned.default_policy())
            for nt in range(warm):
                sim.step(nt)
            torch.cuda.synchronize()
            broyden, gmres = [], []
            t0 = time.perf_counter()
            for nt in range(warm, warm + nsteps):
                b, g = sim.step(nt)
                broyden.append(b)
                gmres.append(g)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            pol = sim.learned_policy()
            r = {"steps_per_s": nsteps / wall, "broyden_iters_per_step": sum(broyden) / nsteps,
                 "gmres_iters_per_step": sum(gmres) / nsteps, "broyden_iters": broyden}
            if label == "learned":
                r["policy"] = {"mode": ["calibrating", "learned", "fell back"][pol.mode],
                               "steps_learned": pol.steps_learned, "steps_plain": pol.steps_plain,
                               "regressions": pol.regressions}
            ref = final_fp64.get(name)
            if ref is not None:
                v = sim.state("body_v").ravel()
                r["swimmer_velocity_error_vs_fp64"] = float(np.linalg.norm(v - ref["body_v"]) /
                                                            np.linalg.norm(ref["body_v"]))
            runs[label] = r
            sim.close()
        out[name] = {"workload": desc, "training_geometry": "same workload, seed 2027",
                     "records": int(records.shape[0]), "collect_s": collect_s,
                     "network": "3 layers, 120 -> 256 -> 256 -> 1000, bf16 weights, FP32 accumulate, rank 4",
                     "train_steps": args.learned_train_steps, "train_s": train_s, "loss_before": loss0,
                     "loss_after": loss1, "loss_last_minibatch": float(losses[-1]) if len(losses) else None,
                     "warmup_steps": warm, "timed_steps": nsteps, **runs,
                     "speedup_learned_vs_plain": runs["learned"]["steps_per_s"] / runs["plain"]["steps_per_s"],
                     "mlp_launches": net.launches}
        net.close()
    return out


def run_batch_accuracy(args, dev, steps: int = 3, tight: float = 1e-7):
    """The per-swimmer error of the uneven-batch workload judged against an
    FP64 oracle: the first ``--accuracy-swimmers`` swimmers of config 4 run
    (a) plain FP64 and (b) FP32C pair sums with FP64 solves, both at the
    benchmark's Broyden tolerance 1e-4, and (c) FP64 at Broyden tolerance
    ``tight`` (GMRES 1e-10), the oracle.  Reports each method's
    per-swimmer velocity error against (c) after ``steps`` steps: both stop
    at a residual of 1e-4, so (a) shows the error the tolerance itself
    leaves, and (b) is on target when it is no larger."""
    from generic_mobility_interface_class_gb300 import workloads
    from generic_mobility_interface_class_gb300.batch import SwimmerBatch
    from generic_mobility_interface_class_gb300._lib import GMI_FP32C, GMI_FP64
    sw = workloads.config4(nswim=args.accuracy_swimmers)
    tight_sw = [dict(kw, tol=tight, linear_tol=1e-10) for kw in sw]
    final = {}
    t0 = time.perf_counter()
    for label, prec, kws in (("fp64", GMI_FP64, sw), ("fp32c", GMI_FP32C, sw), ("oracle", GMI_FP64, tight_sw)):
        with SwimmerBatch(kws, precision=prec, device=dev) as batch:
            batch.prepare()
            for nt in range(steps):
                batch.step(nt)
            final[label] = [a.ravel() for a in batch.state("body_v")]
            if label == "oracle":
                seg_speed = [float(np.sqrt(np.mean(np.sum(a.reshape(-1, 6)[:, :3] ** 2, axis=1))))
                             for a in batch.state("seg_v")]

    def errs(label):
        e = [float(np.linalg.norm(a - o) / np.linalg.norm(o)) for a, o in zip(final[label], final["oracle"])]
        # the same difference against the swimmer's filament speed (translational parts)
        es = [float(np.linalg.norm((a - o).reshape(-1, 6)[:, :3]) / sp)
              for a, o, sp in zip(final[label], final["oracle"], seg_speed)]
        return {"max": max(e), "median": float(np.median(e)), "vs_segment_speed_max": max(es),
                "vs_segment_speed_median": float(np.median(es))}

    return {"swimmers": len(sw), "steps": steps, "broyden_tol": sw[0]["tol"], "oracle_broyden_tol": tight,
            "oracle_gmres_tol": 1e-10, "fp64_vs_oracle": errs("fp64"), "fp32c_vs_oracle": errs("fp32c"),
            "wall_s": time.perf_counter() - t0}


def run_time_steps(args, dev):
    """time-steps/sec of the device time step (gmi_sim_step) on the seeded
    swimmer workloads, plain FP64 against FP32C pair sums with FP64 solves,
    from the same initial state: Broyden tolerance 1e-4, GMRES 1e-8."""
    import torch
    from generic_mobility_interface_class_gb300 import workloads
    from generic_mobility_interface_class_gb300.sim import Simulation
    from generic_mobility_interface_class_gb300._lib import GMI_FP32C, GMI_FP64
    steps_for = dict(kv.split(":") for kv in args.ts_steps.split(",") if kv)
    warm_for = dict(kv.split(":") for kv in getattr(args, "ts_warmups", "").split(",") if kv)
    fp32c_only = {w for w in getattr(args, "ts_fp32c_only", "").split(",") if w}
    out = {}
    for name in [w for w in args.ts_workloads.split(",") if w]:
        w0 = time.perf_counter()
        if name in workloads.BATCH_WORKLOADS:
            warm = int(warm_for.get(name, args.ts_warmup))
            try:
                out[name] = run_batch_time_steps(args, dev, name, int(steps_for.get(name, 3)), warm)
                out[name]["wall_s"] = time.perf_counter() - w0
            except Exception as e:  # keep the rest of the line
                out[name] = {"error": f"{type(e).__name__}: {e}"}
            continue
        desc, make = workloads.WORKLOADS[name]
        kw = make()
        nsteps = int(steps_for.get(name, 10))
        warm = int(warm_for.get(name, args.ts_warmup))
        runs, final = {}, {}
        methods = (("fp32c", GMI_FP32C),) if name in fp32c_only else (("fp64", GMI_FP64), ("fp32c", GMI_FP32C))
        for label, prec in methods:
            sim = Simulation(**kw, precision=prec, device=dev)
            sim.prepare()
            for nt in range(warm):
                sim.step(nt)
            torch.cuda.synchronize()
            l0 = sim.launches
            broyden, gmres = [], []
            with ClockSampler(dev) as clocks:
                t0 = time.perf_counter()
                for nt in range(warm, warm + nsteps):
                    b, g = sim.step(nt)
                    broyden.append(b)
                    gmres.append(g)
                torch.cuda.synchronize()
                wall = time.perf_counter() - t0
            runs[label] = {"warmup_steps": warm, "steps_per_s": nsteps / wall, "ms_per_step": 1e3 * wall / nsteps,
                           "broyden_iters_per_step": sum(broyden) / nsteps, "gmres_iters_per_step": sum(gmres) / nsteps,
                           "broyden_iters": broyden, "gpu_launches": sim.launches - l0, "clocks": clocks.summary()}
            final[label] = {f: sim.state(f).ravel() for f in ("body_v", "seg_v", "seg_q", "body_x")}
            sim.close()

        if "fp64" not in runs:
            out[name] = {"workload": desc, "timed_steps": nsteps, "warmup_steps": warm, "broyden_tol": kw["tol"],
                         "gmres_tol": kw["linear_tol"], **runs, "wall_s": time.perf_counter() - w0,
                         "fp64": "skipped by default (minutes per step); --ts-fp32c-only= measures it"}
            continue

        def rel(f):
            a, b = final["fp64"][f], final["fp32c"][f]
            return float(np.linalg.norm(b - a) / max(np.linalg.norm(a), 1e-300))

        # the swimmer-velocity difference against the filaments' speed: early
        # in a run from a symmetric start the body barely moves, and its own
        # magnitude overstates an error the Broyden tolerance leaves
        seg = final["fp64"]["seg_v"].reshape(-1, 6)[:, :3]
        seg_speed = float(np.sqrt(np.mean(np.sum(seg * seg, axis=1))))
        dvb = final["fp32c"]["body_v"] - final["fp64"]["body_v"]
        body_vs_seg = float(np.linalg.norm(dvb.reshape(-1, 6)[:, :3]) / max(seg_speed, 1e-300))

        if name in ("config3", "config5"):
            final_fp64[name] = final["fp64"]
        out[name] = {"workload": desc, "timed_steps": nsteps, "warmup_steps": warm,
                     "broyden_tol": kw["tol"], "gmres_tol": kw["linear_tol"], **runs,
                     "speedup_fp32c_vs_fp64": runs["fp32c"]["steps_per_s"] / runs["fp64"]["steps_per_s"],
                     "wall_s": time.perf_counter() - w0,
                     "error_fp32c_vs_fp64_after_run": {"swimmer_velocity_rel": rel("body_v"),
                                                       "swimmer_translational_velocity_vs_segment_speed":
                                                           body_vs_seg,
                                                       "segment_velocity_rel": rel("seg_v"),
                                                       "segment_quaternion_rel": rel("seg_q"),
                                                       "body_position_rel": rel("body_x")}}
    return out


def run_batch_time_steps(args, dev, name, nsteps, warmup):
    """Aggregate time-steps/sec of independent swimmers of uneven size
    (batch.SwimmerBatch: one stream and one host thread per swimmer), plain
    FP64 against FP32C pair sums with FP64 solves, and the per-swimmer error
    between the two after the run."""
    import torch
    from generic_mobility_interface_class_gb300 import workloads
    from generic_mobility_interface_class_gb300.batch import SwimmerBatch
    from generic_mobility_interface_class_gb300._lib import GMI_FP32C, GMI_FP64
    desc, make = workloads.BATCH_WORKLOADS[name]
    swimmers = make(nswim=args.ts_swimmers)
    runs, final = {}, {}
    for label, prec in (("fp64", GMI_FP64), ("fp32c", GMI_FP32C)):
        batch = SwimmerBatch(swimmers, precision=prec, device=dev)
        batch.prepare()
        for nt in range(warmup):
            batch.step(nt)
        torch.cuda.synchronize()
        l0 = batch.launches
        broyden, gmres = [], []
        with ClockSampler(dev) as clocks:
            t0 = time.perf_counter()
            for nt in range(warmup, warmup + nsteps):
                it = batch.step(nt)
                broyden.append(sum(b for b, _ in it))
                gmres.append(sum(g for _, g in it))
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        n = len(batch)
        runs[label] = {"swimmer_steps_per_s": n * nsteps / wall, "batch_steps_per_s": nsteps / wall,
                       "ms_per_batch_step": 1e3 * wall / nsteps,
                       "broyden_iters_per_swimmer_step": sum(broyden) / (n * nsteps),
                       "gmres_iters_per_swimmer_step": sum(gmres) / (n * nsteps),
                       "gpu_launches": batch.launches - l0, "clocks": clocks.summary()}
        final[label] = {f: [a.ravel() for a in batch.state(f)] for f in ("body_v", "seg_v")}
        batch.close()

    def rel(f):
        errs = []
        for a, b in zip(final["fp64"][f], final["fp32c"][f]):
            errs.append(float(np.linalg.norm(b - a) / max(np.linalg.norm(a), 1e-300)))
        return {"max": max(errs), "median": float(np.median(errs))}

    def body_vs_seg():
        errs = []
        for a, b, sv in zip(final["fp64"]["body_v"], final["fp32c"]["body_v"], final["fp64"]["seg_v"]):
            sp = float(np.sqrt(np.mean(np.sum(sv.reshape(-1, 6)[:, :3] ** 2, axis=1))))
            errs.append(float(np.linalg.norm((b - a).reshape(-1, 6)[:, :3]) / max(sp, 1e-300)))
        return {"max": max(errs), "median": float(np.median(errs))}

    sizes = [(kw["nblob"], kw["nfil"] * kw["nseg"]) for kw in swimmers]
    if len(swimmers) != 64:
        desc = desc.replace("64 independent", f"{len(swimmers)} independent", 1)
    return {"workload": desc, "swimmers": len(swimmers), "blobs": sum(b for b, _ in sizes),
            "segments": sum(s for _, s in sizes), "host_threads": len(swimmers), "timed_steps": nsteps,
            "warmup_steps": warmup, "broyden_tol": swimmers[0]["tol"], "gmres_tol": swimmers[0]["linear_tol"],
            **runs,
            "speedup_fp32c_vs_fp64": runs["fp32c"]["swimmer_steps_per_s"] / runs["fp64"]["swimmer_steps_per_s"],
            "error_fp32c_vs_fp64_after_run": {"per_swimmer_velocity_rel": rel("body_v"),
                                              "per_swimmer_translational_velocity_vs_segment_speed": body_vs_seg(),
                                              "per_swimmer_segment_velocity_rel": rel("seg_v")}}


def run_gmi(args, world, rank, local):
    import torch
    from generic_mobility_interface_class_gb300 import build as gbuild
    from generic_mobility_interface_class_gb300.mobility import Context
    from generic_mobility_interface_class_gb300._lib import GMI_FP32C, GMI_FP64

    gbuild.build()
    dev = local if torch.cuda.device_count() > 1 else 0
    torch.cuda.set_device(dev)
    prec = GMI_FP32C if args.precision == "fp32c" else GMI_FP64
    x, f = make_inputs(args.n, seed=2026 + rank)
    n = x.shape[0]
    pairs = float(n) * n
    stream = torch.cuda.current_stream()
    ctx = Context(dev, prec, stream)
    xd = torch.as_tensor(x, device="cuda")
    fd = torch.as_tensor(f, device="cuda")
    vd = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    if args.shape:
        tpb_, tt_, sp_, per_ = (int(v) for v in args.shape.split(","))
        ctx.set_shape(0, n, n, tpb_, tt_, sp_, per_)
    elif not args.no_autotune:
        ctx.autotune(0, n, n)
    tpb, tt, splits, tuned = ctx.tuned_shape(0, n, n)
    per_step = ctx.tuned_sources_per_step(0, n, n)
    for _ in range(args.warmup):
        ctx.mss(xd, fd, out=vd)
    ctx.synchronize()

    # ---- device-resident timed region -------------------------------------
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = ctx.launches
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        w0 = time.perf_counter()
        for s in range(args.steps):
            l2_flush.zero_()
            ev[s][0].record(stream)
            ctx.mss(xd, fd, out=vd)
            ev[s][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    barrier(world)
    ctx.synchronize()
    gpu_launches = ctx.launches - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = max_over_ranks(sum(step_ms) / 1e3, world)
    value = world * pairs * args.steps / t_dev
    ms_per_step = 1e3 * t_dev / args.steps

    # ---- end to end through the C ABI with host buffers ----------------------
    xh = torch.as_tensor(x).pin_memory()
    fh = torch.as_tensor(f).pin_memory()
    vh = torch.empty((n, 6), dtype=torch.float64).pin_memory()
    for _ in range(2):
        xd.copy_(xh, non_blocking=True)
        fd.copy_(fh, non_blocking=True)
        ctx.mss(xd, fd, out=vd)
        vh.copy_(vd, non_blocking=True)
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        xd.copy_(xh, non_blocking=True)
        fd.copy_(fh, non_blocking=True)
        ctx.mss(xd, fd, out=vd)
        vh.copy_(vd, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    e2e_value = world * pairs * args.steps / t_e2e

    # ---- accuracy of this precision against the FP64 path ------------------
    extra = {}
    v_main = vd.clone()
    v_main_h = v_main.cpu().numpy()
    v64_h = None
    if not args.no_fp64:
        ctx.set_precision(GMI_FP64)
        ctx.mss(xd, fd, out=vd)  # warm
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.mss(xd, fd, out=vd)
        b.record(stream)
        torch.cuda.synchronize()
        t64 = a.elapsed_time(b) / 1e3
        v64 = vd.clone()
        v64_h = v64.cpu().numpy()
        ctx.set_precision(prec)
        d = (v_main - v64)
        per_t = torch.linalg.norm(d, dim=1) / torch.linalg.norm(v64, dim=1)
        extra["fp64_path"] = {"value": pairs / t64, "unit": "pairs/s", "ms_per_step": 1e3 * t64}
        extra["error_vs_fp64"] = {
            "max_rel_per_target": float(per_t.max()), "rms_rel_per_target": float(torch.sqrt((per_t ** 2).mean())),
            "global_rel": float(torch.linalg.norm(d) / torch.linalg.norm(v64))}
        extra["speedup_vs_fp64_path"] = (pairs / (ms_per_step / 1e3)) / (pairs / t64)

    peak = ctx.fma_peak(prec)
    achieved = FLOP_PER_PAIR_SS * pairs / (ms_per_step / 1e3)
    traffic = PAIR_KERNEL_TRAFFIC.get((n, args.precision, tpb, tt, splits, per_step))
    roofline = {"bound": "fp32" if prec == GMI_FP32C else "fp64",
                "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this shape"
                                   if traffic is not None else "no capture of this launch shape"),
                "algorithmic_bytes": int(n * 48 + n * 48),
                "peak_source": "measured FMA-loop probe on this GPU (gmi_measure_fma_peak)",
                "flops_per_pair": FLOP_PER_PAIR_SS}
    ctx.close()
    time_steps = run_time_steps(args, dev) if args.ts_workloads else {}
    accuracy = {}
    if args.accuracy_swimmers > 0:
        try:
            accuracy = run_batch_accuracy(args, dev)
        except Exception as e:  # keep the rest of the line
            accuracy = {"error": f"{type(e).__name__}: {e}"}
    learned_ab = {}
    if args.learned:
        try:
            learned_ab = run_learned_ab(args, dev)
        except Exception as e:  # keep the rest of the line
            learned_ab = {"error": f"{type(e).__name__}: {e}"}

    line = None
    if rank == 0:
        cpu = None
        try:
            from oracle import rpy
            rpy.build(with_reference=False)
            nt, dt, cores, v_cpu = cpu_sample(x, f, args.cpu_seconds, keep=True)
            cpu = {"value": nt * n / dt, "unit": "pairs/s", "cores": cores, "kind": "port",
                   "sample": f"FP64 oracle, {nt} targets x {n} sources ({dt:.1f} s), OpenMP over targets"}
            # the GPU results on the same targets against the oracle's FP64 sums
            err = {"targets": f"[0, {nt}) of {n}",
                   args.precision: per_target_error(v_main_h[:nt], v_cpu)}
            if v64_h is not None and args.precision != "fp64":
                err["fp64"] = per_target_error(v64_h[:nt], v_cpu)
            extra["error_vs_oracle"] = err
        except Exception as e:  # the baseline is reported, never the measured path
            cpu = {"value": None, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32c" if prec == GMI_FP32C else "f64", "data": "synthetic",
            "config": {"workload": f"RPY apply microbenchmark, N={n} blobs (cube, phi=0.05, min sep 2.2a, "
                                   f"f,tau ~ N(0,1), 6-dof Mss formula, all pairs incl. self)",
                       "n": n, "precision": args.precision, "parallelism": f"replicas x{world}",
                       "launch_shape": {"threads_per_cta": tpb, "targets_per_thread": tt,
                                        "source_splits": splits or "auto", "sources_per_step": per_step,
                                        "autotuned": bool(tuned and not args.shape), "pinned": bool(args.shape)},
                       "l2": "flushed (256 MB write) between timed steps"},
            "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": int(n * 9 * 8),
                    "d2h_bytes_per_step": int(n * 6 * 8), "path": "gmi_Mss_mult with pinned host X,F -> V"},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": gpu_launches,
            "wall_s_timed_region": wall,
            "time_steps": time_steps,
            "learned_initial_inverse_jacobian": learned_ab,
            "config4_accuracy_vs_tight_fp64": accuracy,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gmi(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
