"""Benchmark of the GB300 FAlCon-DNS time step.

Workload (one GPU): the uniform batch of 256 annulus instances sharing the
grid Nr=65, Ntheta=512 (Nm_max=170, Np_max=510), scheme SBDF3 (BDF3/AB3),
dt=1e-6, Pr=1, Ra log-uniform in [1e6, 1e8] (seed 3), noise seeds 1000+k,
amplitude 1e-3, FP64.  A step is one time step of every instance of the
batch.  Metric: instance-steps/s.

Printed as one JSON line by rank 0:
  value        device-resident batched throughput (CUDA events on the
               batch's stream, state resident in HBM; the working set,
               ~1.1 GB, is larger than L2)
  e2e          the same work through the C ABI from host arrays: initial
               state uploaded from pinned host memory, per-step diagnostics
               (writeKE_spectral) read back to the host
  one_at_a_time  the plain path: instances stepped one at a time
  roofline     dominant kernel (by time share) against the measured FP64 FMA
               peak, with the other kernels and launch classes beside it
  cpu_baseline the CPU oracle (OpenMP over modes, as the reference) on a
               bounded sample of the same workload
`--impl reference` times the CPU implementation alone (the reference arm).
Under torchrun each rank runs its own 256-instance shard (weak scaling).
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
sys.path.insert(0, os.path.join(ROOT, "falcon-dns_gb300"))

WORKLOAD = dict(nr=65, nm=170, scheme="SBDF3", dt=1e-6, pr=1.0, n=256, ra_lo=1e6, ra_hi=1e8, ra_seed=3,
                noise_seed0=1000, amp=1e-3)
WORKLOAD_NAME = ("uniform batch of 256 instances, Nr=65, Ntheta=512 (Nm_max=170, Np_max=510), SBDF3, "
                 "dt=1e-6, Pr=1, Ra log-uniform [1e6,1e8], FP64")
METRIC = "instance-steps/s batched+served vs one-at-a-time on same GB300; p50/p99 latency"


def workload_ras(n, rank=0):
    rng = np.random.default_rng(WORKLOAD["ra_seed"] + 7919 * rank)
    u = rng.random(n)
    return [10 ** (6.0 + 2.0 * x) for x in u]


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """The largest x over the ranks of the process group (x itself alone):
    the timed region ends when the slowest rank ends."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, n_per_rank, steps, ms):
    """Instance-steps per second of the whole job: every rank steps its own
    shard of n_per_rank instances `steps` times in `ms` (the max over ranks)."""
    return world * n_per_rank * steps / (ms / 1e3)


def shard(rank, n):
    """Rank `rank`'s instances: Ra values and noise seeds of its own shard."""
    return workload_ras(n, rank), [WORKLOAD["noise_seed0"] + rank * n + k for k in range(n)]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_port_rate(budget_s=10.0, threads=0, rank=0):
    """The CPU oracle on one instance of the workload, all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    if threads:
        oracle.set_threads(threads)
    ra = workload_ras(1, rank)[0]
    s = oracle.Sim(oracle.make_params(WORKLOAD["nr"], WORKLOAD["nm"], WORKLOAD["scheme"], ra=ra,
                                      dt=WORKLOAD["dt"], pr=WORKLOAD["pr"]))
    s.init_noise(WORKLOAD["noise_seed0"], WORKLOAD["amp"])
    s.step(2)  # past the first step, which skips the nonlinear pass
    n = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        s.step(1)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def run_reference(args):
    rank, world, _ = dist_info()
    if world > 1 and rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count()
    ras = workload_ras(4)
    sims = []
    for k, ra in enumerate(ras):
        s = oracle.Sim(oracle.make_params(WORKLOAD["nr"], WORKLOAD["nm"], WORKLOAD["scheme"], ra=ra,
                                          dt=WORKLOAD["dt"], pr=WORKLOAD["pr"]))
        s.init_noise(WORKLOAD["noise_seed0"] + k, WORKLOAD["amp"])
        sims.append(s)
    for k in range(args.warmup):
        sims[k % len(sims)].step(1)
    t0 = time.perf_counter()
    for k in range(args.steps):
        sims[k % len(sims)].step(1)
    dt = time.perf_counter() - t0
    v = args.steps / dt
    line = {
        "metric": METRIC, "value": v, "unit": "instance-steps/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "nr": WORKLOAD["nr"], "nm": WORKLOAD["nm"],
                   "scheme": WORKLOAD["scheme"], "sample": "4 instances of the workload, one time step each per step"},
        "cpu_baseline": {"value": v, "unit": "instance-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} single-instance steps over 4 instances (Nr=65, Nm=170, SBDF3), "
                                   "OpenMP over modes with all host threads"},
        "e2e": {"value": v, "unit": "instance-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


MIXED_NR = (33, 65, 97, 129)
MIXED_NTHETA = (128, 256, 512, 1024, 1536)
MIXED_SCHEMES = ("CNAB2", "SBDF3", "ARS343", "BPR353")
MIXED_PR = (0.1, 1.0, 10.0)


def cfl_dt(nr, nm, eta=0.35):
    """0.2 x the t=0 CFL estimate: the diffusive bounds of get_dtvals
    (src/nonlin.F90:102-104), dr^2 and (r dphi)^2 with dphi = (2/3) pi / Nm,
    times compute_new_dt's Pr factor (src/steptime_rk.F90:194-199), which is
    1 for every Pr."""
    i = np.arange(nr)
    rmin = eta / (1.0 - eta)
    r = rmin + 0.5 * (1.0 + np.cos((nr - 1 - i) * np.pi / (nr - 1)))
    dr = np.empty(nr)
    dr[1:] = r[1:] - r[:-1]
    dr[0] = dr[1]
    rdphi = (2.0 / 3.0) * (r * np.pi) / nm
    return 0.2 * min(float(np.min(dr * dr)), float(np.min(rdphi * rdphi)))


def mixed_requests(fg, n, seed):
    """Instances of the uneven batch / serving stream: Nr from {33,65,97,129},
    Ntheta from {128,...,1536} (Nm = Ntheta // 3), scheme from {CNAB2, SBDF3,
    ARS343, BPR353}, Ra log-uniform in [1e5, 1e8], Pr from {0.1, 1, 10},
    dt = 0.2 x CFL estimate; noise seed per instance."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nr = int(rng.choice(MIXED_NR))
        nm = int(rng.choice(MIXED_NTHETA)) // 3
        scheme = str(rng.choice(MIXED_SCHEMES))
        ra = 10.0 ** rng.uniform(5.0, 8.0)
        pr = float(rng.choice(MIXED_PR))
        p = fg.make_params(nr, nm, scheme, ra=ra, dt=cfl_dt(nr, nm), pr=pr)
        out.append((p, 100000 * seed + k))
    return out


def run_plain(args, fg, stream, torch):
    """The plain reference run: one instance, Nr=33, Ntheta=128 (Nm=42,
    Np=126), CNAB2, dt=1e-5, Ra=1e5, Pr=1, seed 1, stepped alone (its
    latency per step and rate)."""
    p = fg.make_params(33, 42, "CNAB2", ra=1e5, dt=1e-5, pr=1.0)
    it = fg.Instance(p)
    it.set_stream(stream.cuda_stream)
    it.init_noise(1, 1e-3)
    with torch.cuda.stream(stream):
        it.step(gpu_warmup(args))
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = args.plain_steps
    ev0.record(stream)
    it.step(k)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    finite = bool(np.isfinite(it.get_state()["T"]).all())
    it.close()
    return {"value": k / (ms / 1e3), "unit": "instance-steps/s", "steps": k, "ms_per_step": ms / k,
            "state_finite": finite,
            "workload": "one instance Nr=33, Ntheta=128 (Nm=42, Np=126), CNAB2, dt=1e-5, Ra=1e5, Pr=1, seed 1"}


def run_uneven(args, fg, stream, torch):
    """The uneven batch: 512 mixed instances stepped together (one group per
    operator key, groups on concurrent streams, steady steps replayed from
    CUDA graphs)."""
    reqs = mixed_requests(fg, args.uneven_instances, 4)
    t0 = time.perf_counter()
    b = fg.Batch([p for p, _ in reqs])
    setup_s = time.perf_counter() - t0
    b.set_stream(stream.cuda_stream)
    b.init_noise([s for _, s in reqs], 1e-3)
    with torch.cuda.stream(stream):
        b.step(gpu_warmup(args))
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = fg.launch_count()
    ev0.record(stream)
    b.step(args.uneven_steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = fg.launch_count() - l0
    n = len(reqs)
    finite = sum(bool(np.isfinite(b.get_state(i)["T"]).all()) for i in range(n))
    # FLOP of one step of every group from the launch-level model (GEMM,
    # FFT and elementwise counts of each launch), against the step time
    prof = b.profile(1)
    step_flops = sum(v["flops"] for v in prof.values())
    out = {"value": n * args.uneven_steps / (ms / 1e3), "unit": "instance-steps/s", "instances": n,
           "steps": args.uneven_steps, "warmup": gpu_warmup(args), "ms_per_step": ms / args.uneven_steps,
           "operator_groups": b.ngroups, "device_bytes": b.device_bytes, "setup_s": setup_s,
           "gpu_launches": launches, "instances_finite": finite,
           "gflop_per_step": step_flops / 1e9, "tflops": step_flops / (ms / args.uneven_steps / 1e3) / 1e12,
           "classes_serialised_ms": {c: round(v["ms"], 3) for c, v in prof.items()},
           "workload": "512 instances (seed 4): Nr {33,65,97,129}, Ntheta {128,256,512,1024,1536} (Nm=Ntheta//3), "
                       "scheme {CNAB2,SBDF3,ARS343,BPR353}, Ra log-uniform [1e5,1e8], Pr {0.1,1,10}, "
                       "dt = 0.2 x CFL estimate, FP64"}
    b.close()
    return out


def run_single(args, fg, stream, torch):
    """The single larger instance: Nr=97, Ntheta=1024 (Nm=341, Np=1023),
    ARS443, dt=2e-7, Ra=1e8, Pr=1, seed 2; steps of one instance (latency)."""
    p = fg.make_params(97, 341, "ARS443", ra=1e8, dt=2e-7, pr=1.0)
    it = fg.Instance(p)
    it.set_stream(stream.cuda_stream)
    it.init_noise(2, 1e-3)
    with torch.cuda.stream(stream):
        it.step(gpu_warmup(args))
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = args.single_steps
    ev0.record(stream)
    it.step(k)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    prof = it.profile(1)
    flops = sum(v["flops"] for v in prof.values())
    out = {"value": k / (ms / 1e3), "unit": "instance-steps/s", "steps": k, "ms_per_step": ms / k,
           "tflops": flops / (ms / k / 1e3) / 1e12, "state_finite": bool(np.isfinite(it.get_state()["T"]).all()),
           "classes": {c: {"ms_per_step": v["ms"], "launches_per_step": v["launches"]} for c, v in prof.items()},
           "workload": "single instance Nr=97, Ntheta=1024 (Nm=341, Np=1023), ARS443, dt=2e-7, Ra=1e8, Pr=1, seed 2"}
    it.close()
    return out


def run_serving(args, fg, torch):
    """The served stream: Poisson arrivals (50/s, seed 5) of mixed requests,
    admitted by device footprint, stepped by continuous batching; latency is
    submit -> result."""
    rng = np.random.default_rng(5)
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t > args.serve_seconds:
            break
        arrivals.append(t)
    reqs = mixed_requests(fg, len(arrivals), 5)
    lo, hi = 100 * args.serve_horizon_scale, 20000 * args.serve_horizon_scale
    horizons = [max(1, int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))) for _ in reqs]
    srv = fg.Server(args.serve_budget_gb << 30)
    submitted, done_at, ids = 0, {}, {}
    pending = set()
    steps_total = 0
    iters = 0
    t0 = time.perf_counter()
    while len(done_at) < len(reqs):
        now = time.perf_counter() - t0
        while submitted < len(reqs) and arrivals[submitted] <= now:
            p, seed = reqs[submitted]
            ids[srv.submit(p, seed, horizons[submitted])] = submitted
            pending.add(submitted)
            submitted += 1
        if not pending:
            time.sleep(max(0.0, min(arrivals[submitted] - now, 0.01)))
            continue
        srv.iterate()
        iters += 1
        for rid, k in list(ids.items()):
            if k in pending:
                fin, _, _ = srv.poll(rid)
                if fin:
                    done_at[k] = time.perf_counter() - t0
                    pending.discard(k)
                    steps_total += horizons[k]
    wall = time.perf_counter() - t0
    srv.close()
    lat = np.array([done_at[k] - arrivals[k] for k in range(len(reqs))])
    return {"value": steps_total / wall, "unit": "instance-steps/s", "requests": len(reqs),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()), "wall_s": wall, "iterations": iters,
            "instance_steps": steps_total,
            "stream": f"Poisson arrivals {args.serve_rate:g}/s for {args.serve_seconds:g} s (seed 5), requests drawn "
                      f"as the uneven batch, horizons log-uniform [{lo:g}, {hi:g}] steps "
                      f"({args.serve_horizon_scale:g} x [100, 20000]), device budget {args.serve_budget_gb} GB"}


def gpu_warmup(args):
    """Untimed steps before a GPU timing: at least W, and at least 5 so that
    the step graph of every history phase (period <= 4) is captured before
    the timed steps."""
    return max(args.warmup, 5)


# launch class -> kernel function (the operator contractions of the bench's
# groups take the tcgen05 kernel in gemm mode 2, the mma.sync one in mode 1)
def kernel_of_class(c, gemm_mode):
    if c in ("gemm_radial", "gemm_mode_solve"):
        return "tc_gemm_kernel" if gemm_mode >= 2 else "oz_mma_kernel"
    return {"nonlin_fft": "nonlin_kernel", "elementwise": "elementwise kernels"}.get(c, c)


def oz_slice_pairs(nr):
    """bf16 slice products per FP64 product of the operator GEMMs (N >= 16
    columns each, contraction length K = Nr): 7-bit slices, 9 per operand and
    the 45 pairs s + t <= 8, when K padded to 16 is at most 112; else 6-bit
    slices, 10 per operand and the 55 pairs s + t <= 9."""
    return 45 if (nr + 15) // 16 * 16 <= 112 else 55


def tensor_peak():
    """Measured bf16 dense peak (TFLOP/s) for a kernel timed inside a long
    step (the sustained figure), with where it came from."""
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["bf16_tflops_sustained"]), "bf16_tflops_sustained of measured MEASURED_PEAKS.json"
    except (OSError, ValueError, KeyError):
        return 1700.0, "fallback 1.7 PFLOP/s sustained bf16"


def load_traffic(kernel):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(path))
        return d.get(kernel)
    except (OSError, ValueError):
        return None


def run_gpu(args):
    import torch
    import falcon_gpu as fg
    import build as falcon_build

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    falcon_build.build()
    fg.lib()
    stream = torch.cuda.Stream()
    fg.set_gemm_mode(args.gemm_mode)
    if args.uneven_only:  # profiling captures of the uneven batch
        if rank == 0:
            print(json.dumps({"uneven_batch": run_uneven(args, fg, stream, torch)}), flush=True)
        return
    W = WORKLOAD
    n = args.instances or W["n"]
    ras, seeds = shard(rank, n)
    params = [fg.make_params(W["nr"], W["nm"], W["scheme"], ra=ra, dt=W["dt"], pr=W["pr"]) for ra in ras]
    peak = fg.fp64_peak_gflops()
    mma_peak = fg.fp64_mma_peak_gflops()

    # ---- device-resident batched throughput ----
    b = fg.Batch(params)
    b.set_stream(stream.cuda_stream)
    b.init_noise(seeds, W["amp"])
    with torch.cuda.stream(stream):
        b.step(gpu_warmup(args))
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = fg.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        b.step(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = fg.launch_count() - launches0
    ms = max_over_ranks(ms, world, "cuda")
    value = whole_job_rate(world, n, args.steps, ms)
    finite = all(np.isfinite(b.get_state(i)["T"]).all() for i in (0, n - 1))

    # ---- kernel classes (CUDA events per launch on the same stream) ----
    ngroups = b.ngroups
    prof = b.profile(3)
    tot = sum(v["ms"] for v in prof.values())
    # the launch classes by kernel function: both GEMM classes are launches
    # of oz_mma_kernel (with the slicing of their X columns)
    kern = {}
    for c, v in prof.items():
        k = kernel_of_class(c, args.gemm_mode)
        e = kern.setdefault(k, {"ms": 0.0, "flops": 0.0, "launches": 0.0, "traffic_sum": 0.0, "traffic_ok": True})
        e["ms"] += v["ms"]; e["flops"] += v["flops"]; e["launches"] += v["launches"]
        t = load_traffic(c)
        if t is None:
            e["traffic_ok"] = False
        else:
            # profiles/traffic.json holds bytes per call of a 128-instance
            # group; a call here covers one group of n / ngroups instances
            e["traffic_sum"] += t * (n / ngroups) / 128.0 * v["launches"]
    dom = max(kern, key=lambda k: kern[k]["ms"])

    tpeak, tpeak_src = tensor_peak()

    def kernel_roof(k):
        e = kern[k]
        ach = e["flops"] / (e["ms"] / 1e3) / 1e12
        r = {"bound": "fp64", "achieved": ach, "peak": peak / 1e3, "frac": ach / (peak / 1e3), "share": e["ms"] / tot,
             "launches_per_step": e["launches"] / 3,
             "traffic": (e["traffic_sum"] / e["launches"]) if (e["traffic_ok"] and e["launches"]) else None}
        if k in ("oz_mma_kernel", "tc_gemm_kernel"):
            # bf16 slice products executed per second against the tensor
            # peak; the FP64-equivalent rate against the DFMA peak beside it
            pairs = oz_slice_pairs(W["nr"])
            r.update({"bound": "tensor", "achieved": ach * pairs, "peak": tpeak,
                      "frac": ach * pairs / tpeak, "peak_source": tpeak_src, "slice_pairs": pairs,
                      "fp64_equivalent_tflops": ach, "fp64_equivalent_over_dfma_peak": ach / (peak / 1e3),
                      "note": ("the kernel slices its X columns in shared memory" if k == "tc_gemm_kernel" else
                               "time includes the per-call slicing of the X columns (oz_slice_cols_kernel)")})
        return r
    d = kernel_roof(dom)
    achieved = d["achieved"]
    roofline = {"bound": d["bound"], "achieved": achieved, "peak": d["peak"], "unit": "TFLOP/s",
                "frac": d["frac"], "traffic": d["traffic"], "kernel": dom,
                "share": d["share"],
                "kernels": {k: kernel_roof(k) for k in kern},
                "peak_source": d.get("peak_source", "FP64 FMA throughput measured live by the library's DFMA "
                                                    "kernel (no FP64 figure in MEASURED_PEAKS.json)"),
                "fp64_mma_peak_tflops": mma_peak / 1e3,
                "classes": {k: {"ms_per_step": v["ms"] / 3, "tflops": v["flops"] / (v["ms"] / 1e3) / 1e12,
                                "share": v["ms"] / tot, "launches_per_step": v["launches"] / 3}
                            for k, v in prof.items()}}
    b.close()

    # ---- end to end through the C ABI from host arrays ----
    e2e = None
    if not args.uniform_only:
        b2 = fg.Batch(params)
        b2.set_stream(stream.cuda_stream)
        # host initial conditions (Fortran layout), pinned
        b2.init_noise(seeds, W["amp"])
        # every instance's four fields back to back in one pinned buffer each
        init_T = np.concatenate([b2.get_state(i)["T"].ravel() for i in range(n)])
        host = [torch.from_numpy(init_T).pin_memory().numpy()]
        host += [torch.zeros(init_T.shape, dtype=torch.complex128).pin_memory().numpy() for _ in range(3)]
        torch.cuda.synchronize()
        k_e2e = max(10, args.steps // 2)
        h2d = d2h = 0
        t0 = time.perf_counter()
        b2.set_states(*host)
        h2d += sum(a.nbytes for a in host)
        for k in range(k_e2e):
            b2.step(1)
            diag = b2.diagnostics_array()  # writeKE_spectral every step (n_KE = 1, the namelist default)
            d2h += n * 8 * 8
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": world * n * k_e2e / e2e_s, "unit": "instance-steps/s",
               "h2d_bytes_per_step": h2d // k_e2e, "d2h_bytes_per_step": d2h // k_e2e,
               "steps": k_e2e, "diagnostics_every": 1,
               "note": "C-ABI calls from the host: initial fields (T, omega, u_phi, u_r) of every instance uploaded "
                       "from pinned host arrays inside the timed region (falcon_batch_set_states), one "
                       "falcon_batch_step per step, and the step's "
                       "diagnostics (KE, Nusselt, power of every instance) read back every step"}
        b2.close()

    # ---- plain one-instance-at-a-time GPU path ----
    n1 = 0 if args.uniform_only else min(args.one_at_a_time, n)
    insts = []
    for k in range(n1):
        it = fg.Instance(params[k])
        it.set_stream(stream.cuda_stream)
        it.init_noise(seeds[k], W["amp"])
        insts.append(it)
    for it in insts:
        it.step(gpu_warmup(args))
    torch.cuda.synchronize()
    k1 = max(5, args.steps // 4)
    ev0.record(stream)
    for k in range(k1):
        for it in insts:
            it.step(1)
    ev1.record(stream)
    torch.cuda.synchronize()
    one_rate = n1 * k1 / (ev0.elapsed_time(ev1) / 1e3) if n1 else None
    for it in insts:
        it.close()

    uneven = serving = plain = single = None
    if not args.uniform_only:
        plain = run_plain(args, fg, stream, torch)
        single = run_single(args, fg, stream, torch)
    if not args.no_mixed and not args.uniform_only:
        uneven = run_uneven(args, fg, stream, torch)
        serving = run_serving(args, fg, torch)

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return
    cpu = None
    if not args.no_cpu:
        rate, nst, secs = cpu_port_rate(args.cpu_seconds)
        rate1, nst1, secs1 = cpu_port_rate(args.cpu_seconds, threads=1)
        cpu = {"value": rate, "unit": "instance-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{nst} time steps of one workload instance (Nr=65, Nm=170, SBDF3) in {secs:.1f} s, "
                         "CPU oracle with OpenMP over modes on all host threads",
               "one_thread": {"value": rate1, "unit": "instance-steps/s", "cores": 1,
                              "sample": f"{nst1} time steps in {secs1:.1f} s, OMP_NUM_THREADS=1"}}
    line = {
        "metric": METRIC, "value": value, "unit": "instance-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": gpu_warmup(args), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "instances_per_gpu": n, "nr": W["nr"], "nm": W["nm"],
                   "np": 3 * W["nm"], "scheme": W["scheme"], "dt": W["dt"],
                   "l2": "working set ~1.1 GB per GPU, larger than L2 (129 MB); no flush needed",
                   "parallelism": f"replicas x{world}",
                   "groups_per_gpu": ngroups,
                   "groups": "the instances run as groups of at most 128 sharing the operators, one stream each "
                             "(falcon_set_max_group_size default), so one group's nonlinear pass overlaps "
                             "another's contractions; the roofline classes time the groups one after another"},
        "e2e": e2e,
        "plain_reference_run": plain,
        "single_instance": single,
        "uneven_batch": uneven,
        "serving": serving,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "gemm_mode": {4: "autotuned: per contraction shape the fastest measured of FP64 FMA, mma.sync slices and "
                         "tcgen05 slices (tensor memory accumulators), measured at the first warm-up step",
                      3: "tcgen05 for every sliced contraction",
                      2: "fixed rules: tcgen05 for contractions that fill the GPU, mma.sync below, FMA under 16 columns",
                      1: "mma.sync", 0: "FP64 FMA"}[args.gemm_mode],
        "tuned_shapes": fg.tune_entries()[0],
        "state_finite": bool(finite),
        # last, so that a reader of the line's tail sees the target ratio
        "one_at_a_time": {"value": one_rate, "unit": "instance-steps/s", "instances": n1, "steps": k1},
        "batched_over_one_at_a_time": (value / world / one_rate) if one_rate else None,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--instances", type=int, default=0, help="instances per GPU (default 256)")
    ap.add_argument("--one-at-a-time", dest="one_at_a_time", type=int, default=16)
    ap.add_argument("--cpu-seconds", dest="cpu_seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", dest="no_cpu", action="store_true")
    ap.add_argument("--no-mixed", dest="no_mixed", action="store_true", help="skip the uneven batch and serving")
    ap.add_argument("--uneven-only", dest="uneven_only", action="store_true",
                    help="the uneven batch alone (profiling captures)")
    ap.add_argument("--uniform-only", dest="uniform_only", action="store_true",
                    help="the uniform batch alone (profiling captures): no e2e, one-at-a-time, plain, single, mixed")
    ap.add_argument("--single-steps", dest="single_steps", type=int, default=200)
    ap.add_argument("--plain-steps", dest="plain_steps", type=int, default=500)
    ap.add_argument("--gemm-mode", dest="gemm_mode", type=int, default=4, choices=[0, 1, 2, 3, 4],
                    help="operator contractions: 4 autotuned per shape (FMA / mma.sync / tcgen05), 3 tcgen05, "
                         "2 fixed rules, 1 mma.sync slices, 0 FP64 FMA")
    ap.add_argument("--uneven-instances", dest="uneven_instances", type=int, default=512)
    ap.add_argument("--uneven-steps", dest="uneven_steps", type=int, default=500)
    ap.add_argument("--serve-rate", dest="serve_rate", type=float, default=50.0)
    ap.add_argument("--serve-seconds", dest="serve_seconds", type=float, default=15.0)
    ap.add_argument("--serve-horizon-scale", dest="serve_horizon_scale", type=float, default=0.15)
    ap.add_argument("--serve-budget-gb", dest="serve_budget_gb", type=int, default=64)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
