"""Benchmark of the Gravity-Sim force-and-integrate path on GB300.

Headline workload: Barnes-Hut, N = 500,000 spiral galaxy (exponential disk, scale 30,
r <= 100, two-arm logarithmic spiral, pitch 15 deg, amplitude 0.3, circular velocities
from the enclosed mass + 5% dispersion, masses U[1,10]), softening 0.2, dt = 1e-3,
seeded synthetic input, gated at <= 1e-3 RMS relative force error against the FP64
direct sum at every measured step: accurate mode (bounding box, quadrupoles, safe opening
radius, group walk) with the relative opening criterion, alpha = 0.006 with a theta floor
of 0.2; a step without a previous |a| (the first, and every end-to-end step, since an
upload forgets |a|) first estimates |a| by a walk at theta = 1.  Beside it: the same
accurate mode with the geometric criterion alone at theta = 0.3, and the reference's own
opening rule at theta = 1 (fixed +-500 box, monopoles, warp vote) with its error; the
latter does not meet the gate.  A step is one simulation step of the whole system.

  value  particle-steps/s, device time (CUDA events on the simulation's stream), state
         resident in HBM; L2 flushed (256 MiB write) before every timed step
  e2e    the same metric through the C ABI with host buffers: every step uploads the
         state from pinned host memory (gs_set_particles), runs one step (gs_run) and
         reads the state back (gs_get_particles), host wall clock
  roofline  the traversal kernel: algorithmic FLOP of the accepted interactions
         (14 per monopole, 33 per quadrupole) over its CUDA-event time, against the
         FP32 FMA rate
  direct_config  direct sum, N = 4096 uniform disk at rest, 10 steps (its own roofline,
           error and CPU baseline)
  batched  512 systems of uneven N stepped together, against each run alone
  served   a Poisson stream of simulation requests through the serving loop, against the
           plain path taking them one at a time (p50 / p99 latency)
  direct_precision_study  N=50k direct sum over 1000 steps: Kahan-compensated against
           plain FP32 sums, force error against FP64 and energy drift

Multi-GPU: independent replicas (the path has no exchange step), one per rank.
`--impl reference` times the CPU restatement of the reference's algorithm (oracle/,
all host threads) on the same workload; it loads nothing of the library.
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
ACCURATE = 0x70  # GS_FLAGS_ACCURATE
RELATIVE = 0x100  # GS_FLAG_RELATIVE_MAC
DIRECT_SUM, BARNES_HUT = 0, 1  # gs_algorithm
BOX_FIXED, BOX_BOUNDING = 0, 1  # gs_box_mode
GEN_UNIFORM_DISK, GEN_SPIRAL, GEN_EXP_DISK_COLLISION = 16, 17, 18  # gs_generate_type
ERROR_SAMPLE = 16384  # particles whose FP64 force the gated error is measured on
# DRAM bytes of one launch of the traversal kernel on a workload, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum), and that launch's algorithmic bytes
FORCE_CAPTURE = {
    "bh500k": {"traffic": 55.191040e6 + 1.843712e6, "algorithmic": 49.034368e6},
}


def workloads():
    spiral = dict(algo=BARNES_HUT, gen=GEN_SPIRAL, n=500000, size=100.0, seed=2002)
    return {
        "bh500k": dict(spiral, box=BOX_BOUNDING, theta=1.0, alpha=0.006, floor=0.2, flags=ACCURATE | RELATIVE,
                       oracle_flags=15,
                       desc="Barnes-Hut N=500000 spiral galaxy, accurate mode (bounding box, quadrupole, safe "
                            "radius, 64-particle group walk), relative opening criterion alpha=0.006 with "
                            "theta floor 0.2 (|a| estimated by a theta=1 walk where none is known), softening "
                            "0.2, dt=1e-3"),
        "bh500k-theta": dict(spiral, box=BOX_BOUNDING, theta=0.3, flags=ACCURATE, oracle_flags=7,
                             desc="Barnes-Hut N=500000 spiral galaxy, accurate mode (bounding box, quadrupole, "
                                  "safe radius, 64-particle group walk), geometric criterion theta=0.3, "
                                  "softening 0.2, dt=1e-3"),
        "bh500k-30bit": dict(spiral, box=BOX_BOUNDING, theta=1.0, alpha=0.006, floor=0.2, flags=ACCURATE | RELATIVE,
                             oracle_flags=15, key_bits=15,
                             desc="the headline workload with 15 bits per axis: 30-bit bounding-box Morton keys "
                                  "(4 radix passes, 16 tree levels)"),
        "bh500k-reference-rule": dict(spiral, box=BOX_FIXED, theta=1.0, flags=0, oracle_flags=0,
                                      desc="Barnes-Hut N=500000 spiral galaxy, the reference's opening rule "
                                           "(fixed +-500 box, monopoles, warp vote) theta=1, softening 0.2, dt=1e-3"),
        "direct4096": dict(algo=DIRECT_SUM, gen=GEN_UNIFORM_DISK, n=4096, size=100.0, seed=1001, box=0,
                           theta=1.0, flags=0, oracle_flags=0, steps=10,
                           desc="direct sum N=4096 uniform disk r=100 at rest, masses U[1,10], softening 0.2, "
                                "dt=1e-3, 10 steps"),
        "direct50k": dict(algo=DIRECT_SUM, gen=GEN_EXP_DISK_COLLISION, n=50000, size=100.0, seed=1003,
                          box=0, theta=1.0, flags=0, oracle_flags=0,
                          desc="direct sum N=50000 two exponential disks at (+-50,0), v=(0,+-3)"),
    }


class NvmlClockSampler:
    """SM clock and clock-event (throttle) reasons read through NVML every millisecond
    during the timed region (read-only queries; the timed region of a default run lasts
    about 10 ms, too short for nvidia-smi's 200 ms sampling)."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device, period_s=0.001):
        import ctypes as C
        self.C = C
        self.nvml = C.CDLL("libnvidia-ml.so.1")
        if self.nvml.nvmlInit_v2() != 0:
            raise OSError("nvmlInit_v2 failed")
        self.h = C.c_void_p()
        if self.nvml.nvmlDeviceGetHandleByIndex_v2(C.c_uint(device), C.byref(self.h)) != 0:
            raise OSError("nvmlDeviceGetHandleByIndex_v2 failed")
        fn = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn or self.nvml.nvmlDeviceGetCurrentClocksThrottleReasons
        self.period = period_s
        self.samples = []
        self.stop_flag = threading.Event()

    def _one(self):
        C = self.C
        clk, mx, rs = C.c_uint(0), C.c_uint(0), C.c_ulonglong(0)
        if self.nvml.nvmlDeviceGetClockInfo(self.h, 1, C.byref(clk)) != 0:  # NVML_CLOCK_SM
            return None
        self.nvml.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx))
        self.reasons_fn(self.h, C.byref(rs))
        return clk.value, mx.value, rs.value

    def _run(self):
        while not self.stop_flag.is_set():
            s = self._one()
            if s:
                self.samples.append(s)
            time.sleep(self.period)

    def start(self):
        s = self._one()  # one sample at the start, then the polling thread
        if s:
            self.samples.append(s)
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def stop(self):
        self.stop_flag.set()
        self.t.join(timeout=2)
        s = self._one()
        if s:
            self.samples.append(s)
        self.nvml.nvmlShutdown()
        if not self.samples:
            return None
        reasons = set()
        for _, _, r in self.samples:
            reasons.update(nm for bit, nm in self.REASONS.items() if r & bit)
        return {"sm_mhz": float(np.median([c for c, _, _ in self.samples])),
                "sm_max_mhz": float(max(m for _, m, _ in self.samples)), "samples": len(self.samples),
                "reasons": sorted(reasons), "source": "NVML, every 1 ms"}


def clock_sampler(device):
    try:
        return NvmlClockSampler(device)
    except (OSError, AttributeError):
        return ClockSampler(device)


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


def dist_setup(backend="nccl"):
    """Ranks from torchrun's environment: one replica per GPU (every rank steps its own
    system; no data-path collective), NCCL for the timing barrier and reductions.  The
    gloo backend serves the CPU tests of this logic."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist, local):
    if dist is None:
        return
    if dist.get_backend() == "nccl":
        dist.barrier(device_ids=[local])
    else:
        dist.barrier()


def reduce_op(dist, x, op):
    """max or sum of x over the ranks (x itself on one rank)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def job_value(dist, particles, steps, dev_ms):
    """Whole-job particle-steps/s: the particles of every rank over the slowest rank's time."""
    return reduce_op(dist, float(particles), "sum") * steps / (reduce_op(dist, dev_ms, "max") / 1e3)


def make_params(gsim, wl, local, flags):
    return gsim.default_params(algorithm=wl["algo"], box_mode=wl["box"], accuracy_parameter=wl["theta"],
                               relative_accuracy=wl.get("alpha", 0.0), relative_theta_floor=wl.get("floor", 0.0),
                               key_bits=wl.get("key_bits", 0), device=local, flags=wl["flags"] | flags)


def autotune(gsim, wl, local, steps=10):
    """The launch-shape autotuner (gs_tune_shape) on the workload's own system; systems of
    this key created afterwards get the shape it picks."""
    r = gsim.tune_shape(make_params(gsim, wl, local, 0), wl["n"], generator=wl["gen"], seed=wl["seed"], steps=steps)
    return {"shape": r.best.as_dict(), "ms_per_step": r.best_ms, "default_shape_ms_per_step": r.default_ms,
            "candidates_timed": int(r.candidates)}


def step_errors(gsim, params, pos, vel, mass, sub, steps, warm=0):
    """Relative force error against the FP64 direct sum on the particles `sub`, for each
    of `steps` consecutive steps after `warm` unmeasured ones, from a new system holding
    the given state (so the first step is one without a previous |a|).  FP64 forces of
    each step's starting state come from a direct-sum system holding that state
    (gs_accel_f64)."""
    p = gsim.Params.from_buffer_copy(params)
    p.flags |= gsim.FLAG_RECORD_ACCEL
    d = gsim.default_params(algorithm=gsim.DIRECT_SUM, device=p.device)
    errs = []
    with gsim.Simulation(pos, vel, mass, params=p) as es:
        if warm:
            es.run(warm)
        for _ in range(steps):
            start = es.get_particles()
            es.run(1)
            acc = es.get_accel()[sub].astype(np.float64)
            with gsim.Simulation(*start, params=d) as fs:
                a64 = fs.accel_f64(sub)
            errs.append(np.linalg.norm(acc - a64, axis=1) / np.maximum(np.linalg.norm(a64, axis=1), 1e-30))
    return errs


def error_summary(errs):
    """RMS of each step, the worst (the gated figure), and median / p99 / max over all."""
    rms = [float(np.sqrt(np.mean(e ** 2))) for e in errs]
    e = np.concatenate(errs)
    return {"rms": max(rms), "rms_per_step": rms, "median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)),
            "max": float(e.max())}


def interaction_counts(gsim, wl, pos, vel, mass, local):
    """Tree and interaction counts of the second step (the first with a previous |a|),
    from a separate simulation built with GS_FLAG_COUNT_INTERACTIONS (the counting
    kernels are not the timed ones)."""
    if wl["algo"] != gsim.BARNES_HUT:
        return {}
    with gsim.Simulation(pos, vel, mass, params=make_params(gsim, wl, local, gsim.FLAG_COUNT_INTERACTIONS)) as cs:
        cs.run(2)
        st = cs.stats()
        return {"interactions": int(st.interactions), "tests": int(st.warp_visits),
                "tree_records": int(st.tree_records), "internal_nodes": int(st.internal_nodes),
                "node_interactions": int(st.node_interactions)}


def stage_times(gsim, wl, pos, vel, mass, local, steps):
    """Per-stage milliseconds per step from a separate run with GS_FLAG_PROFILE (stage
    events inside the step graph; they also turn the overlapped launches off, so the
    timed run does not use this flag)."""
    with gsim.Simulation(pos, vel, mass, params=make_params(gsim, wl, local, gsim.FLAG_PROFILE)) as ps:
        ps.run(3)
        ps.sync()
        ps.reset_stats()
        ps.run(steps)
        ps.sync()
        st = ps.stats()
        return {nm: st.stage_ms[i] / st.stage_launches[i] for i, nm in enumerate(gsim.STAGES) if st.stage_launches[i]}


def measure(gsim, torch, wl, pos, vel, mass, args, local, dist, sample_clocks):
    """Device-timed steps with an L2 flush before each (the state stays resident)."""
    sim = gsim.Simulation(pos, vel, mass, params=make_params(gsim, wl, local, 0))
    stream = torch.cuda.ExternalStream(sim.stream(), device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    sim.run(args.warmup)
    sim.sync()
    sim.reset_stats()
    launches0 = sim.stats().kernel_launches
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = clock_sampler(local) if sample_clocks else None
    barrier(dist, local)
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # L2 flush: 256 MiB written before every timed step
            starts[k].record(stream)
            sim.run(1)
            ends[k].record(stream)
    sim.sync()
    torch.cuda.synchronize()
    barrier(dist, local)
    clk = clocks.stop() if clocks else None
    st = sim.stats()
    dev_ms = float(sum(s.elapsed_time(e) for s, e in zip(starts, ends)))
    out = {"dev_ms": dev_ms, "launches": int(st.kernel_launches - launches0), "clocks": clk, "sim": sim,
           "stage_ms": stage_times(gsim, wl, pos, vel, mass, local, max(3, args.steps))}
    out.update(interaction_counts(gsim, wl, pos, vel, mass, local))
    return out


BATCH_DESC = ("512 independent systems, N log-uniform in [1024, 262144] (seed 1004), each a uniform disk "
              "(r=100) or a spiral galaxy with p=0.5; direct sum (Kahan FP32) below the tuned crossover N, "
              "Barnes-Hut accurate mode (%s) above it; softening 0.2, dt=1e-3")


def batch_specs(count=512, seed=1004, lo=1024, hi=262144):
    rng = np.random.default_rng(seed)
    n = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(np.int64)
    kind = np.where(rng.random(count) < 0.5, GEN_UNIFORM_DISK, GEN_SPIRAL)
    return [(int(k), int(x), seed * 1000 + j) for j, (k, x) in enumerate(zip(kind, n))]


def batch_params(gsim, local, n, crossover, theta, alpha, floor=0.0, flags=0):
    """Direct sum below the crossover; above it accurate-mode Barnes-Hut with the relative
    criterion (alpha > 0, with its theta floor; theta for steps without a previous |a|) or
    theta alone (alpha = 0)."""
    if n < crossover:
        return gsim.default_params(algorithm=gsim.DIRECT_SUM, device=local, flags=flags)
    return gsim.default_params(algorithm=gsim.BARNES_HUT, box_mode=gsim.BOX_BOUNDING, accuracy_parameter=theta,
                               relative_accuracy=alpha, relative_theta_floor=floor, device=local,
                               flags=ACCURATE | (RELATIVE if alpha > 0 else 0) | flags)


def bh_mode_desc(theta, alpha, floor=0.0):
    return (f"relative criterion alpha={alpha:g} with theta floor {floor or theta:g}, theta={theta:g} without a "
            f"previous |a|" if alpha > 0 else f"theta={theta:g}")


def measure_batched(gsim, torch, args, local):
    """Config of many systems: the batched path (one launch per stage, a CUDA graph per
    step) against the plain path run one system at a time (gs_run of each system in turn,
    each with its own step graph), both timed with CUDA events on the device."""
    t_setup = time.perf_counter()
    d = gsim.default_params(algorithm=gsim.DIRECT_SUM, device=local)
    theta, alpha, floor = args.batch_theta, args.batch_alpha, args.batch_floor
    h = batch_params(gsim, local, 1 << 30, 0, theta, alpha, floor)
    tune = gsim.tune_crossover(d, h, min_n=1024, max_n=262144, particles_per_probe=1 << 21, seed=4000)
    xo = tune["crossover"]
    specs = batch_specs()
    sims = []
    for kind, n, seed in specs:
        pos, vel, mass = gsim.generate(kind, n, size=100.0, seed=seed)
        sims.append(gsim.Simulation(pos, vel, mass, params=batch_params(gsim, local, n, xo, theta, alpha, floor)))
    total_n = float(sum(n for _, n, _ in specs))
    n_bh = sum(1 for _, n, _ in specs if n >= xo)
    setup_s = time.perf_counter() - t_setup
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    steps = args.batch_steps

    batch = gsim.Batch(sims)
    stream = torch.cuda.ExternalStream(batch.stream, device=local)
    batch.run(args.warmup)
    batch.sync()
    tb = batch.tune(steps=3) if not args.no_tune else None  # the batched kernels' launch shape
    tuned = {"shape": tb.best.as_dict(), "ms_per_step": tb.best_ms, "default_shape_ms_per_step": tb.default_ms,
             "candidates_timed": int(tb.candidates)} if tb else None
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.zero_()  # L2 flush before every timed batched step
            starts[k].record(stream)
            batch.run(1)
            ends[k].record(stream)
    batch.sync()
    torch.cuda.synchronize()
    wall_b = time.perf_counter() - w0
    dev_b = float(sum(s.elapsed_time(e) for s, e in zip(starts, ends))) / 1e3
    kps = batch.kernels_per_step
    batch.close()

    # plain path, one system at a time: warm (graph capture), then `steps` steps each
    dev_p = 0.0
    w0 = time.perf_counter()
    for s in sims:
        s.run(args.warmup)
        s.sync()
        st = torch.cuda.ExternalStream(s.stream(), device=local)
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st):
            flush.zero_()  # each system starts cold, as when it runs on its own
            a.record(st)
            s.run(steps)
            z.record(st)
        s.sync()
        dev_p += a.elapsed_time(z) / 1e3
    wall_p = time.perf_counter() - w0  # includes the warm-up steps

    # force error of a stratified sample of members, from each one's current state (after
    # all the steps above): the first step has no previous |a| (it estimates it), the
    # second opens nodes by the |a| the first left
    errs = _member_errors(gsim, local, specs, sims, xo, theta, alpha, floor)
    for s in sims:
        s.close()
    value = total_n * steps / dev_b
    plain = total_n * steps / dev_p
    return {"workload": BATCH_DESC % bh_mode_desc(theta, alpha, floor), "theta": theta, "alpha": alpha,
            "theta_floor": floor, "value": value, "unit": "particle-steps/s", "steps": steps,
            "ms_per_step": dev_b * 1e3 / steps, "systems": len(specs), "particles": int(total_n),
            "barnes_hut_systems": n_bh, "direct_systems": len(specs) - n_bh, "crossover_n": xo, "tuning": tune,
            "kernels_per_step": kps, "gpu_launches": kps * steps, "autotuned": tuned,
            "plain_one_at_a_time": {"value": plain, "device_s": dev_p, "wall_s_incl_warmup": wall_p},
            "speedup_vs_plain": value / plain, "wall_value": total_n * steps / wall_b,
            "force_error_sample": errs, "force_error_worst_rms": max(e["rms"] for e in errs), "setup_s": setup_s,
            "l2": "flushed (256 MiB write) before every timed batched step and before each plain system"}


def _member_errors(gsim, local, specs, sims, xo, theta, alpha, floor, per_kind=12, sample=4096, steps=2):
    """Force error of `per_kind` Barnes-Hut members of each generator type (evenly spread
    over their sizes) and two direct-sum members, on `sample` particles each, at `steps`
    steps from the member's current state."""
    chosen = []
    for kind in (GEN_UNIFORM_DISK, GEN_SPIRAL):
        idx = sorted((j for j, (k, n, _) in enumerate(specs) if k == kind and n >= xo), key=lambda j: specs[j][1])
        if idx:
            chosen += [idx[int(q)] for q in np.unique(np.linspace(0, len(idx) - 1, per_kind).round())]
    small = sorted((j for j, (_, n, _) in enumerate(specs) if n < xo), key=lambda j: specs[j][1])
    chosen += [small[0], small[-1]] if small else []
    rng = np.random.default_rng(1)
    out = []
    for j in sorted(set(chosen)):
        kind, n, _ = specs[j]
        pos, vel, mass = sims[j].get_particles()
        sub = rng.choice(n, min(sample, n), replace=False).astype(np.uint32)
        errs = step_errors(gsim, batch_params(gsim, local, n, xo, theta, alpha, floor), pos, vel, mass, sub, steps)
        r = error_summary(errs)
        out.append({"n": n, "kind": "spiral" if kind == GEN_SPIRAL else "uniform disk",
                    "algorithm": "barnes-hut" if n >= xo else "direct", "rms": r["rms"],
                    "rms_per_step": r["rms_per_step"], "max": r["max"], "subsample": int(len(sub))})
    return out


SERVE_DESC = ("Poisson stream (mean 200 requests/s, seed 1005) of simulation requests: N log-uniform in "
              "[2048, 1048576], steps uniform in [10, 1000], generator uniform over uniform disk / spiral galaxy / "
              "two-disk collision; direct sum below the tuned crossover, Barnes-Hut accurate mode (%s) above; "
              "150 GB device-memory budget; softening 0.2, dt=1e-3")


def serve_trace(count, seed=1005, rate=200.0, lo=2048, hi=1 << 20):
    import gsim

    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, count)
    arrivals = np.cumsum(gaps) - gaps[0]
    n = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(np.int64)
    steps = rng.integers(10, 1001, count)
    gen = rng.choice([GEN_UNIFORM_DISK, GEN_SPIRAL, GEN_EXP_DISK_COLLISION], count)
    reqs = [gsim.make_request(int(n[j]), int(steps[j]), int(gen[j]), seed=seed * 100000 + j) for j in range(count)]
    return reqs, arrivals


def _latency_summary(lat):
    lat = np.asarray(lat)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max())}


def measure_served(gsim, torch, args, local, crossover, theta, alpha, floor):
    """The served workload through gs_server (continuous batching, admission by device
    footprint), and the plain sequential path on the same trace: each request in arrival
    order, generated, created, run with gs_run and read back, one at a time."""
    reqs, arrivals = serve_trace(args.serve_requests)
    d = gsim.default_params(algorithm=gsim.DIRECT_SUM, device=local)
    b = batch_params(gsim, local, 1 << 30, 0, theta, alpha, floor)
    work = float(sum(r.particle_count * r.steps for r in reqs))
    with gsim.Server(150 * 10 ** 9, crossover, d, b, max_resident_particles=args.serve_max_particles,
                     steps_in_flight=2, policy=gsim.SERVE_FIFO) as srv:
        t0 = srv.clock()
        ids = srv.run_trace(reqs, arrivals, timeout_s=1800)
        info = [srv.request(i) for i in ids]
        st = srv.stats()
    lat = [x.finish_s - x.arrival_s for x in info]
    makespan = max(x.finish_s for x in info) - (t0 + float(arrivals[0]))
    served = {"value": work / makespan, "makespan_s": makespan, "latency": _latency_summary(lat),
              "queue_wait": _latency_summary([x.admit_s - x.arrival_s for x in info]),
              "batched_steps": st["batched_steps"], "plan_changes": st["plan_changes"],
              "peak_memory_gb": st["peak_memory_in_use"] / 1e9,
              "peak_resident_particles": st["peak_resident_particles"], "failed": st["failed"]}

    served["gpu_busy_s"] = st["gpu_busy_seconds"]
    served["gpu_busy_fraction"] = st["gpu_busy_seconds"] / makespan

    # plain sequential path: one request at a time in arrival order, real-time arrivals;
    # where its time goes, per phase (host wall clock; the steps also in device time)
    lat_p = []
    bd = dict(wait_for_arrival_s=0.0, generate_s=0.0, create_and_upload_s=0.0, steps_wall_s=0.0,
              steps_device_s=0.0, readback_s=0.0, destroy_s=0.0)
    start = time.perf_counter()
    for r, a in zip(reqs, arrivals):
        now = time.perf_counter() - start
        if now < a:
            time.sleep(a - now)
            bd["wait_for_arrival_s"] += a - now
        t0 = time.perf_counter()
        pos, vel, mass = gsim.generate(r.generator, r.particle_count, size=r.generate_size, seed=r.seed)
        t1 = time.perf_counter()
        sim = gsim.Simulation(pos, vel, mass, params=d if r.particle_count < crossover else b)
        t2 = time.perf_counter()
        stream = torch.cuda.ExternalStream(sim.stream(), device=local)
        ea, ez = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            ea.record(stream)
            sim.run(r.steps)
            ez.record(stream)
        sim.sync()
        t3 = time.perf_counter()
        sim.get_particles()
        t4 = time.perf_counter()
        sim.close()
        t5 = time.perf_counter()
        bd["generate_s"] += t1 - t0
        bd["create_and_upload_s"] += t2 - t1
        bd["steps_wall_s"] += t3 - t2
        bd["steps_device_s"] += ea.elapsed_time(ez) / 1e3
        bd["readback_s"] += t4 - t3
        bd["destroy_s"] += t5 - t4
        lat_p.append(time.perf_counter() - start - a)
    makespan_p = time.perf_counter() - start - float(arrivals[0])
    plain = {"value": work / makespan_p, "makespan_s": makespan_p, "latency": _latency_summary(lat_p),
             "breakdown": bd, "gpu_busy_fraction": bd["steps_device_s"] / makespan_p}
    # the served path is GPU-bound when its device time fills its makespan; then no
    # scheduling can beat plain makespan / served device time on this trace
    served["speedup_ceiling_at_its_gpu_time"] = makespan_p / max(st["gpu_busy_seconds"], 1e-9)
    served["force_error_sample"] = _request_errors(gsim, reqs, d, b, crossover)
    served["force_error_worst_rms"] = max(e["rms"] for e in served["force_error_sample"])
    return {"workload": SERVE_DESC % bh_mode_desc(theta, alpha, floor), "requests": len(reqs), "theta": theta,
            "alpha": alpha, "theta_floor": floor, "crossover_n": crossover,
            "particle_steps": work, "value": served["value"], "unit": "particle-steps/s", "served": served,
            "plain_sequential": plain, "speedup_vs_plain": served["value"] / plain["value"],
            "max_resident_particles": args.serve_max_particles, "policy": "fifo with conservative backfill"}


def _request_errors(gsim, reqs, d, b, crossover, per_kind=2, sample=4096, steps=3):
    """Force error of served requests: `per_kind` requests of each generator type (the
    smallest and the largest Barnes-Hut ones of the trace), each stepped alone from its
    generated state with the served parameters -- a served request ends bit-identical to
    the same system run alone -- on `sample` particles at each of its first `steps` steps."""
    names = {GEN_UNIFORM_DISK: "uniform disk", GEN_SPIRAL: "spiral", GEN_EXP_DISK_COLLISION: "two-disk collision"}
    rng = np.random.default_rng(2)
    out = []
    for kind in names:
        rs = sorted((r for r in reqs if r.generator == kind and r.particle_count >= crossover),
                    key=lambda r: r.particle_count)
        for r in ([rs[0], rs[-1]] if len(rs) > 1 else rs)[:per_kind]:
            n = r.particle_count
            pos, vel, mass = gsim.generate(r.generator, n, size=r.generate_size, seed=r.seed)
            sub = rng.choice(n, min(sample, n), replace=False).astype(np.uint32)
            res = error_summary(step_errors(gsim, b, pos, vel, mass, sub, steps))
            out.append({"n": n, "kind": names[kind], "rms": res["rms"], "rms_per_step": res["rms_per_step"],
                        "max": res["max"], "subsample": int(len(sub))})
    return out


PREC_DESC = ("direct sum N=50000, two exponential disks (scale length 20, truncated at r <= 50) centred at "
             "(+-50, 0) with bulk velocities (0, +-3) and circular speeds inside each disk, masses U[1,10], "
             "softening 0.2, dt=1e-3, 1000 steps (seed 1003)")


def precision_study(gsim, torch, args, local, steps=1000, every=100, sample=2048):
    """Direct-sum precision study: the same 1000-step run with Kahan-compensated FP32 tile
    sums (the default), with plain FP32 tile sums, and with the shader's plain sequential
    FP32 sum (REFERENCE math).  Every `every` steps: relative force error of the step
    against the FP64 direct sum on a fixed subsample, and the FP64 energy drift."""
    n = 50000
    pos, vel, mass = gsim.generate(gsim.GEN_EXP_DISK_COLLISION, n, size=100.0, seed=1003)
    sub = np.random.default_rng(3).choice(n, sample, replace=False).astype(np.uint32)
    variants = (("kahan_fp32", gsim.MATH_FAST, 0),
                ("plain_fp32_tiles", gsim.MATH_FAST, gsim.FLAG_PLAIN_SUM),
                ("plain_fp32_sequential_reference_math", gsim.MATH_REFERENCE, 0))
    out = {}
    for name, mm, fl in variants:
        p = gsim.default_params(algorithm=gsim.DIRECT_SUM, math_mode=mm, device=local, flags=fl | gsim.FLAG_RECORD_ACCEL)
        with gsim.Simulation(pos, vel, mass, params=p) as sim:
            ke, pe = sim.energy_f64()
            e0 = ke + pe
            rms, mx, drift = [], [], []
            for k in range(0, steps, every):
                a64 = sim.accel_f64(sub)  # FP64 forces of the current state
                sim.run(1)                # the FP32 step from that state records its forces
                acc = sim.get_accel()[sub].astype(np.float64)
                e = np.linalg.norm(acc - a64, axis=1) / np.maximum(np.linalg.norm(a64, axis=1), 1e-300)
                rms.append(float(np.sqrt(np.mean(e ** 2))))
                mx.append(float(e.max()))
                sim.run(every - 1)
                ke, pe = sim.energy_f64()
                drift.append(abs((ke + pe) - e0) / abs(e0))
            # device time per step of the same variant, state resident
            stream = torch.cuda.ExternalStream(sim.stream(), device=local)
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            sim.sync()
            with torch.cuda.stream(stream):
                a.record(stream)
                sim.run(20)
                z.record(stream)
            sim.sync()
            ms = a.elapsed_time(z) / 20
        out[name] = {"force_error_rms_max_over_checkpoints": max(rms), "force_error_rms_mean": float(np.mean(rms)),
                     "force_error_max": max(mx), "energy_drift_final": drift[-1], "energy_drift_max": max(drift),
                     "ms_per_step": ms, "checkpoint_rms": rms}
    return {"workload": PREC_DESC, "steps": steps, "checkpoint_every": every, "subsample": sample,
            "energy": "FP64 kinetic + softened potential (gs_energy_f64), drift = |E(t) - E(0)| / |E(0)|",
            "variants": out}


def force_error(gsim, wl, pos, vel, mass, local, steps=5):
    """Relative force error against the FP64 direct sum (GPU FP64 kernel) on a
    16384-particle subsample, at each of the first `steps` steps from the generated state
    (the first has no previous |a|): the RMS of the worst step (the gated figure), each
    step's RMS, and median / p99 / max over all."""
    sub = np.random.default_rng(0).choice(wl["n"], min(ERROR_SAMPLE, wl["n"]), replace=False).astype(np.uint32)
    r = error_summary(step_errors(gsim, make_params(gsim, wl, local, 0), pos, vel, mass, sub, steps))
    r.update(subsample=int(len(sub)), steps=f"steps 1..{steps} from the generated state")
    return r


def force_algorithmic_bytes(wl, m):
    """Bytes the traversal kernel must move once per launch: tree records (16 B each), the
    moments and child links of internal records (32 B each), the particle state read and
    written (32 B per particle), the sorted key and order (8 B) and the previous and new
    |a| (8 B) per particle."""
    n_al = (wl["n"] + 63) // 64 * 64
    amag = 8 if wl["flags"] & RELATIVE else 0
    return 16 * m["tree_records"] + 32 * m["internal_nodes"] + (32 + 8 + amag) * n_al


def roofline_of(gsim, wl, m, capture=None):
    """FP32 roofline of the force kernel.  `capture`: DRAM bytes of one launch of the same
    kernel on the same workload from an ncu capture, with the algorithmic bytes of that
    launch; the line's traffic is that figure scaled to this run's algorithmic bytes."""
    algorithmic = None
    if wl["algo"] == BARNES_HUT:
        t = m["stage_ms"]["force"] / 1e3
        # 14 FLOP per monopole interaction (particle leaves; every record under the
        # reference rule), 33 per quadrupole interaction (accurate-mode nodes)
        quads = m["node_interactions"] if wl["flags"] & 0x10 else 0
        flops = 14.0 * (m["interactions"] - quads) + 33.0 * quads
        achieved = flops / t / 1e12
        algorithmic = force_algorithmic_bytes(wl, m)
        extra = {"kernel": "k_force_group" if wl["flags"] & 0x40 else "k_force",
                 "interactions_per_step": m["interactions"], "quadrupole_interactions_per_step": quads,
                 "tests_per_step": m["tests"], "tree_records": m["tree_records"],
                 "internal_nodes": m["internal_nodes"], "algorithmic_bytes": algorithmic,
                 "flop_model": "14 FLOP per monopole (leaf) interaction, 33 per quadrupole (node) interaction "
                               "(FMA = 2); interactions of both walks of a step that estimates |a| are counted"}
    else:
        t = m["stage_ms"]["direct"] / 1e3
        n_al = (wl["n"] + 63) // 64 * 64
        achieved = 14.0 * n_al * n_al / t / 1e12
        extra = {"kernel": "k_direct_fast", "pairs_per_step": n_al * n_al, "flop_model": "14 FLOP per pair"}
    traffic = source = None
    if capture and algorithmic:
        traffic = capture["traffic"] * algorithmic / capture["algorithmic"]
        source = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this kernel on this workload "
                  f"({capture['traffic'] / 1e6:.2f} MB at {capture['algorithmic'] / 1e6:.2f} MB algorithmic), "
                  f"scaled by this run's algorithmic bytes; ncu cannot run inside the timed bench")
    r = {"bound": "fp32", "achieved": achieved, "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
         "frac": achieved / FP32_NOMINAL_TFLOPS, "traffic": traffic, "traffic_source": source,
         "peak_source": "nominal FP32 FMA rate at 2070 MHz (MEASURED_PEAKS.json has no FP32 figure)",
         "stage_ms_per_step": m["stage_ms"]}
    r.update(extra)
    return r


def _cpu_bh_step_seconds(oracle, wl, pos, vel, mass, threads, budget):
    """Seconds of one Barnes-Hut step of the oracle on `threads` threads: the second step
    of the system (a full first step leaves every particle's |a|), with the force walk
    sampled (every k-th group, its time scaled by k) when a full step would exceed the
    budget.  Returns (seconds, stride)."""
    st = oracle.State(pos, vel, mass)
    kw = dict(box_mode=wl["box"], theta=wl["theta"], keep_tree=False, threads=threads, flags=wl["oracle_flags"],
              rel_alpha=wl.get("alpha", 0.0), rel_floor=wl.get("floor"))
    r = oracle.bh_step(st, **kw)  # the full first step (time estimate of the second)
    stride = max(1, int(np.ceil((r["build_seconds"] + r["walk_seconds"]) / budget)))
    r = oracle.bh_step(st, walk_stride=stride, **kw)
    return r["build_seconds"] + stride * r["walk_seconds"], stride


def cpu_baseline(wl, pos, vel, mass, seconds_budget=15.0):
    """The CPU restatement (oracle/) of one step of the same workload, on all host threads
    and on one core; a long Barnes-Hut force walk is sampled."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    out = {}
    for cores in (threads, 1):
        if wl["algo"] == BARNES_HUT:
            t, stride = _cpu_bh_step_seconds(oracle, wl, pos, vel, mass, cores, seconds_budget)
            sample = (f"1 step of the same {wl['n']}-particle system (the second, after a full first step): tree "
                      f"build on 1 thread, force walk on {cores} thread(s)" +
                      (f" over every {stride}-th group of 64, its time scaled by {stride}" if stride > 1 else ""))
        else:
            st = oracle.State(pos, vel, mass)
            t0 = time.perf_counter()
            oracle.direct_step(st, threads=cores)
            t = time.perf_counter() - t0
            sample = f"1 step of the same {wl['n']}-particle system on {cores} thread(s)"
        out[cores] = {"value": wl["n"] / t, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                      "sample": sample}
    r = dict(out[threads])
    r["single_core"] = out[1]
    return r


def direct_config(gsim, torch, args, local):
    """Direct sum, N = 4096 uniform disk at rest, 10 steps: device time per step (CUDA
    events, L2 flushed before each step), FP32 roofline, force error of every step
    against the FP64 direct sum on all particles, and the CPU baseline."""
    wl = dict(workloads()["direct4096"], name="direct4096")
    pos, vel, mass = gsim.generate(wl["gen"], wl["n"], size=wl["size"], seed=wl["seed"])
    steps = wl["steps"]
    tuned = autotune(gsim, wl, local) if not args.no_tune else None
    p = make_params(gsim, wl, local, 0)
    with gsim.Simulation(pos, vel, mass, params=p) as sim:
        stream = torch.cuda.ExternalStream(sim.stream(), device=local)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
        times = []
        for rep in range(args.warmup + 1):  # warm-up runs of the 10 steps, then the timed one
            sim.set_particles(pos, vel, mass)
            sim.sync()
            starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            with torch.cuda.stream(stream):
                for k in range(steps):
                    flush.zero_()
                    starts[k].record(stream)
                    sim.run(1)
                    ends[k].record(stream)
            sim.sync()
            times = [a.elapsed_time(b) for a, b in zip(starts, ends)]
        dev_ms = float(sum(times))
    err = error_summary(step_errors(gsim, p, pos, vel, mass, np.arange(wl["n"], dtype=np.uint32), steps))
    m = {"stage_ms": {"direct": dev_ms / steps}}
    return {"workload": wl["desc"], "value": wl["n"] * steps / (dev_ms / 1e3), "unit": "particle-steps/s",
            "steps": steps, "ms_per_step": dev_ms / steps, "roofline": roofline_of(gsim, wl, m),
            "force_error_vs_fp64": dict(err, subsample=wl["n"], steps="steps 1..10 from the generated state"),
            "cpu_baseline": cpu_baseline(wl, pos, vel, mass), "autotuned": tuned,
            "l2": "flushed (256 MiB write) before every timed step"}


def run_reference(args, wl):
    """--impl reference: the CPU restatement of the reference's algorithm, all host threads,
    on inputs from the oracle's own generators (nothing of the library is loaded)."""
    from oracle import oracle

    world = int(os.environ.get("WORLD_SIZE", "1"))
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    pos, vel, mass = oracle.generate(wl["gen"], wl["n"], size=wl["size"], seed=wl["seed"])
    threads = os.cpu_count() or 1
    st = oracle.State(pos, vel, mass)
    budget = 150.0 / max(1, args.steps + args.warmup)  # whole run within a few minutes
    stride, times = 1, []
    kw = dict(box_mode=wl["box"], theta=wl["theta"], keep_tree=False, threads=threads, flags=wl["oracle_flags"],
              rel_alpha=wl.get("alpha", 0.0), rel_floor=wl.get("floor"))
    for k in range(args.warmup + args.steps):
        if wl["algo"] == BARNES_HUT:
            if k == 0:  # a full step: time estimate, and every particle's |a| for the next
                r = oracle.bh_step(st, **kw)
                t = r["build_seconds"] + r["walk_seconds"]
                stride = max(1, int(np.ceil(t / budget)))
                continue
            r = oracle.bh_step(st, walk_stride=stride, **kw)
            t = r["build_seconds"] + stride * r["walk_seconds"]
        else:
            t0 = time.perf_counter()
            oracle.direct_step(st, threads=threads)
            t = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(t)
    tot = float(np.sum(times))
    value = wl["n"] * len(times) / tot
    sample = (f"each step: full tree build + force walk of every {stride}-th group of 64, walk time scaled by "
              f"{stride}" if wl["algo"] == BARNES_HUT and stride > 1 else "each step: one full step of the system")
    out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "impl": "reference", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded generator)",
           "config": {"workload": wl["desc"], "particles_per_gpu": wl["n"], "parallelism": f"replicas x{world}"},
           "l2": "n/a (CPU)",
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
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the reference-rule theta=1 line")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-system batched line")
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--batch-theta", type=float, default=1.0,
                    help="theta of the batched and served Barnes-Hut systems (the |a| estimate of a step "
                         "without a previous |a|)")
    ap.add_argument("--batch-floor", type=float, default=0.2,
                    help="theta floor of the relative criterion of the batched and served systems")
    ap.add_argument("--batch-alpha", type=float, default=0.006,
                    help="relative criterion alpha of the batched and served Barnes-Hut systems (0: theta alone)")
    ap.add_argument("--no-served", action="store_true", help="skip the served (request stream) line")
    ap.add_argument("--no-precision", action="store_true", help="skip the direct-sum precision study")
    ap.add_argument("--no-direct-config", action="store_true", help="skip the N=4096 direct-sum line")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner (default shapes)")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serve-max-particles", type=int, default=0, help="resident particle cap (0: budget only)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    wl = dict(workloads()[args.workload], name=args.workload)
    if args.impl == "reference":
        return run_reference(args, wl)

    import build as pkg_build

    pkg_build.build()
    import gsim
    import torch

    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    pos, vel, mass = gsim.generate(wl["gen"], wl["n"], size=wl["size"], seed=wl["seed"] + rank)
    tuned = autotune(gsim, wl, local) if not args.no_tune else None
    m = measure(gsim, torch, wl, pos, vel, mass, args, local, dist, sample_clocks=True)
    sim = m.pop("sim")
    max_ms = reduce_op(dist, m["dev_ms"], "max")
    total_particles = reduce_op(dist, float(wl["n"]), "sum")
    value = job_value(dist, wl["n"], args.steps, m["dev_ms"])

    # end to end through the C ABI with pinned host buffers
    import ctypes as C

    e2e_steps = args.e2e_steps or args.steps
    hp = torch.from_numpy(pos).pin_memory().numpy()
    hv = torch.from_numpy(vel).pin_memory().numpy()
    hm = torch.from_numpy(mass).pin_memory().numpy()
    op_ = torch.empty((wl["n"], 2), dtype=torch.float32).pin_memory().numpy()
    ov_ = torch.empty((wl["n"], 2), dtype=torch.float32).pin_memory().numpy()
    om_ = torch.empty((wl["n"],), dtype=torch.float32).pin_memory().numpy()
    L = gsim.lib()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    barrier(dist, local)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gsim._check(L.gs_set_particles(sim.handle, fp(hp), fp(hv), fp(hm)))
        gsim._check(L.gs_run(sim.handle, 1))
        gsim._check(L.gs_get_particles(sim.handle, fp(op_), fp(ov_), fp(om_)))
    e2e_s = reduce_op(dist, time.perf_counter() - t0, "max")
    e2e = {"value": total_particles * e2e_steps / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": int(hp.nbytes + hv.nbytes + hm.nbytes),
           "d2h_bytes_per_step": int(op_.nbytes + ov_.nbytes + om_.nbytes), "steps": e2e_steps}
    sim.close()

    err = force_error(gsim, wl, pos, vel, mass, local) if rank == 0 else None
    secondary = theta_only = keys30 = None
    if rank == 0 and world == 1 and args.workload == "bh500k" and not args.no_secondary:
        lines = []
        for name in ("bh500k-theta", "bh500k-30bit", "bh500k-reference-rule"):
            wl2 = dict(workloads()[name], name=name)
            m2 = measure(gsim, torch, wl2, pos, vel, mass, args, local, None, sample_clocks=False)
            m2.pop("sim").close()
            lines.append({"workload": wl2["desc"], "value": wl2["n"] * args.steps / (m2["dev_ms"] / 1e3),
                          "ms_per_step": m2["dev_ms"] / args.steps, "stage_ms_per_step": m2["stage_ms"],
                          "interactions_per_step": m2.get("interactions"),
                          "force_error_vs_fp64": force_error(gsim, wl2, pos, vel, mass, local)})
        theta_only, keys30, secondary = lines
    batched = served = None
    if rank == 0 and world == 1 and not args.no_batched:
        batched = measure_batched(gsim, torch, args, local)
    if rank == 0 and world == 1 and not args.no_served:
        xo = batched["crossover_n"] if batched else 2500
        served = measure_served(gsim, torch, args, local, xo, args.batch_theta, args.batch_alpha, args.batch_floor)
    precision = None
    if rank == 0 and world == 1 and not args.no_precision:
        precision = precision_study(gsim, torch, args, local)
    direct = None
    if rank == 0 and world == 1 and not args.no_direct_config:
        direct = direct_config(gsim, torch, args, local)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, pos, vel, mass)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
               "config": {"workload": wl["desc"], "particles_per_gpu": wl["n"], "parallelism": f"replicas x{world}"},
               "l2": "flushed (256 MiB write) before every timed step",
               "e2e": e2e, "gpu_launches": m["launches"] * world,
               "roofline": roofline_of(gsim, wl, m, FORCE_CAPTURE.get(args.workload)),
               "cpu_baseline": cpu, "force_error_vs_fp64": err, "clocks": m["clocks"],
               "autotuned": tuned, "accurate_theta_only": theta_only, "keys_30bit": keys30,
               "reference_rule_theta1": secondary, "direct_config": direct,
               "batched": batched, "served": served, "direct_precision_study": precision}
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
