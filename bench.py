"""Benchmark of the Gravity-Sim force-and-integrate path on GB300.

Default workload: Barnes-Hut, N = 500,000 spiral galaxy (exponential disk, scale 30,
r <= 100, two-arm logarithmic spiral, pitch 15 deg, amplitude 0.3, circular velocities
from the enclosed mass + 5% dispersion, masses U[1,10]), theta = 1, softening 0.2,
dt = 1e-3, seeded synthetic input.  A step is one simulation step of the whole system.

  value  particle-steps/s, device time (CUDA events on the simulation's stream), state
         resident in HBM; L2 flushed (256 MiB write) before every timed step
  e2e    the same metric through the C ABI with host buffers: every step uploads the
         state from pinned host memory (gs_set_particles), runs one step (gs_run) and
         reads the state back (gs_get_particles), host wall clock
  roofline  the traversal kernel: 14 FLOP per accepted (particle, record) interaction
         over its CUDA-event time, against the FP32 FMA peak

Multi-GPU: independent replicas (the path has no exchange step), one per rank.
`--impl reference` times the CPU restatement of the reference's algorithm (oracle/,
all host threads) on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gravity-sim_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-steps/s (BH N=500k; batched/served vs plain) at <=1e-3 rel force err"
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12  # 152 SMs x 128 FP32 lanes x FMA at 2070 MHz


def workloads():
    import gsim

    return {
        "bh500k": dict(algo=gsim.BARNES_HUT, gen=gsim.GEN_SPIRAL, n=500000, size=100.0, theta=1.0, seed=2002,
                       desc="Barnes-Hut N=500000 spiral galaxy, theta=1, softening 0.2, dt=1e-3"),
        "direct4096": dict(algo=gsim.DIRECT_SUM, gen=gsim.GEN_UNIFORM_DISK, n=4096, size=100.0, theta=1.0,
                           seed=1001, desc="direct sum N=4096 uniform disk r=100, softening 0.2, dt=1e-3"),
        "direct50k": dict(algo=gsim.DIRECT_SUM, gen=gsim.GEN_EXP_DISK_COLLISION, n=50000, size=100.0, theta=1.0,
                          seed=1003, desc="direct sum N=50000 two exponential disks at (+-50,0), v=(0,+-3)"),
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist, local):
    if dist is not None:
        import torch

        dist.barrier(device_ids=[local])


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline(wl, box, pos, vel, mass, seconds_budget=30.0):
    """The CPU restatement (oracle/) on all host threads, one step of the same workload;
    the force walk is sampled (every k-th warp) when a full step would exceed the budget."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    st = oracle.State(pos, vel, mass)
    if wl["algo"] == 1:
        r = oracle.bh_step(st, box_mode=box, theta=wl["theta"], keep_tree=False, threads=threads, walk_stride=8)
        est = r["build_seconds"] + 8 * r["walk_seconds"]
        stride = max(1, int(np.ceil(est / seconds_budget)))
        st = oracle.State(pos, vel, mass)
        r = oracle.bh_step(st, box_mode=box, theta=wl["theta"], keep_tree=False, threads=threads, walk_stride=stride)
        t = r["build_seconds"] + stride * r["walk_seconds"]
        sample = (f"1 step of the same {wl['n']}-particle system: full tree build, force walk of every "
                  f"{stride}-th warp of 32 (walk time scaled by {stride})")
    else:
        t0 = time.perf_counter()
        oracle.direct_step(st, threads=threads)
        t = time.perf_counter() - t0
        sample = f"1 step of the same {wl['n']}-particle system"
    return {"value": wl["n"] / t, "unit": "particle-steps/s", "cores": threads, "kind": "port", "sample": sample}


def run_reference(args, wl, box):
    """--impl reference: the CPU restatement of the reference's algorithm, all host threads."""
    import gsim
    from oracle import oracle

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    pos, vel, mass = gsim.generate(wl["gen"], wl["n"], size=wl["size"], seed=wl["seed"])
    threads = os.cpu_count() or 1
    st = oracle.State(pos, vel, mass)
    budget = 150.0 / max(1, args.steps + args.warmup)  # whole run within a few minutes
    stride = 1
    times = []
    for k in range(args.warmup + args.steps):
        if wl["algo"] == 1:
            r = oracle.bh_step(st, box_mode=box, theta=wl["theta"], keep_tree=False, threads=threads,
                               walk_stride=stride)
            t = r["build_seconds"] + stride * r["walk_seconds"]
            if k == 0:
                stride = max(1, int(np.ceil(t / budget)))
        else:
            t0 = time.perf_counter()
            oracle.direct_step(st, threads=threads)
            t = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(t)
    tot = float(np.sum(times))
    value = wl["n"] * len(times) / tot
    sample = (f"each step: full tree build + force walk of every {stride}-th warp, walk time scaled by {stride}"
              if wl["algo"] == 1 and stride > 1 else "each step: one full step of the system")
    out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "impl": "reference", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded generator)",
           "config": {"workload": wl["desc"] + f" ({'fixed box' if box == 0 else 'bounding box'})",
                      "particles": wl["n"], "steps": "bench steps", "l2": "n/a (CPU)"},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bh500k")
    ap.add_argument("--box", default="fixed", choices=["fixed", "bbox"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: same as --steps")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    import gsim

    wl = workloads()[args.workload]
    box = gsim.BOX_FIXED_500 if args.box == "fixed" else gsim.BOX_BOUNDING
    if args.impl == "reference":
        return run_reference(args, wl, box)

    import build as pkg_build

    pkg_build.build()
    import torch

    world, rank, local, dist = dist_setup(args)
    torch.cuda.set_device(local)
    pos, vel, mass = gsim.generate(wl["gen"], wl["n"], size=wl["size"], seed=wl["seed"] + rank)
    flags = gsim.FLAG_PROFILE | (gsim.FLAG_COUNT_INTERACTIONS if wl["algo"] == gsim.BARNES_HUT else 0)
    params = gsim.default_params(algorithm=wl["algo"], box_mode=box, accuracy_parameter=wl["theta"], device=local,
                                 flags=flags)
    sim = gsim.Simulation(pos, vel, mass, params=params)
    stream = torch.cuda.ExternalStream(sim.stream(), device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    # warm-up (untimed)
    sim.run(args.warmup)
    sim.sync()
    sim.reset_stats()
    launches0 = sim.stats().kernel_launches

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier(dist, local)
    torch.cuda.synchronize()
    clocks.start()
    inter_total = 0
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # L2 flush: 256 MiB written before every timed step
            starts[k].record(stream)
            sim.run(1)
            ends[k].record(stream)
    sim.sync()
    torch.cuda.synchronize()
    barrier(dist, local)
    clk = clocks.stop()
    st = sim.stats()
    dev_ms = float(sum(s.elapsed_time(e) for s, e in zip(starts, ends)))
    launches = st.kernel_launches - launches0
    max_ms = reduce_max(dist, dev_ms)
    total_particles = reduce_sum(dist, float(wl["n"]))
    value = total_particles * args.steps / (max_ms / 1e3)

    # roofline of the dominant kernel (per-stage CUDA events recorded inside the step graph)
    stage_ms = {nm: st.stage_ms[i] for i, nm in enumerate(gsim.STAGES) if st.stage_launches[i]}
    stage_n = {nm: st.stage_launches[i] for i, nm in enumerate(gsim.STAGES) if st.stage_launches[i]}
    if wl["algo"] == gsim.BARNES_HUT:
        kern = "force"
        t_launch = stage_ms["force"] / stage_n["force"] / 1e3
        flops = 14.0 * st.interactions  # interactions of the last step ~ per launch
        achieved = flops / t_launch / 1e12
        extra = {"interactions_per_step": int(st.interactions), "warp_visits_per_step": int(st.warp_visits),
                 "tree_records": int(st.tree_records), "internal_nodes": int(st.internal_nodes)}
    else:
        kern = "direct"
        t_launch = stage_ms["direct"] / stage_n["direct"] / 1e3
        n_al = sim.n_al
        achieved = 14.0 * n_al * n_al / t_launch / 1e12
        extra = {"pairs_per_step": n_al * n_al}
    roofline = {"kernel": kern, "bound": "fp32", "achieved": achieved, "peak": FP32_NOMINAL_TFLOPS,
                "unit": "TFLOP/s", "frac": achieved / FP32_NOMINAL_TFLOPS, "traffic": None,
                "peak_source": "nominal FP32 FMA rate at 2070 MHz (MEASURED_PEAKS.json has no FP32 figure)",
                "stage_ms_per_step": {k: v / stage_n[k] for k, v in stage_ms.items()}}
    roofline.update(extra)

    # end to end through the C ABI with pinned host buffers
    e2e_steps = args.e2e_steps or args.steps
    hp = torch.from_numpy(pos).pin_memory().numpy()
    hv = torch.from_numpy(vel).pin_memory().numpy()
    hm = torch.from_numpy(mass).pin_memory().numpy()
    op = torch.empty((wl["n"], 2), dtype=torch.float32).pin_memory().numpy()
    ov = torch.empty((wl["n"], 2), dtype=torch.float32).pin_memory().numpy()
    om = torch.empty((wl["n"],), dtype=torch.float32).pin_memory().numpy()
    import ctypes as C

    L = gsim.lib()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    barrier(dist, local)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        gsim._check(L.gs_set_particles(sim.handle, fp(hp), fp(hv), fp(hm)))
        gsim._check(L.gs_run(sim.handle, 1))
        gsim._check(L.gs_get_particles(sim.handle, fp(op), fp(ov), fp(om)))
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(dist, e2e_s)
    e2e = {"value": total_particles * e2e_steps / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": int(hp.nbytes + hv.nbytes + hm.nbytes),
           "d2h_bytes_per_step": int(op.nbytes + ov.nbytes + om.nbytes), "steps": e2e_steps}

    # force error of the fast path against the FP64 direct sum (4096-particle subsample)
    err = None
    if rank == 0:
        p2 = gsim.default_params(algorithm=wl["algo"], box_mode=box, accuracy_parameter=wl["theta"], device=local,
                                 flags=gsim.FLAG_RECORD_ACCEL)
        with gsim.Simulation(pos, vel, mass, params=p2) as es:
            es.run(1)
            acc = es.get_accel().astype(np.float64)
            es.set_particles(pos, vel, mass)
            sub = np.random.default_rng(0).choice(wl["n"], min(4096, wl["n"]), replace=False).astype(np.uint32)
            a64 = es.accel_f64(sub)
        e = np.linalg.norm(acc[sub] - a64, axis=1) / np.maximum(np.linalg.norm(a64, axis=1), 1e-30)
        err = {"rms": float(np.sqrt(np.mean(e ** 2))), "median": float(np.median(e)),
               "p99": float(np.quantile(e, 0.99)), "max": float(e.max()), "subsample": int(len(sub))}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, box, pos, vel, mass)

    sim.close()
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
               "config": {"workload": wl["desc"] + f" ({'fixed box +-500' if box == 0 else 'bounding box'})",
                          "particles_per_gpu": wl["n"], "parallelism": f"replicas x{world}",
                          "l2": "flushed (256 MiB write) before every timed step"},
               "e2e": e2e, "gpu_launches": int(launches) * world, "roofline": roofline, "cpu_baseline": cpu,
               "force_error_vs_fp64": err, "clocks": clk}
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
