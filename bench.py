"""Benchmark of the GB300 DEM step: particle-steps/s on the batched-colonies
workload (256 colonies, log-uniform 500..50 000 spheres, FP32 pair math),
with the plain FP64 form on the same workload beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload colonies|sphere_fp32|sphere_plain|rod_trees]
                  [--precision fp32f|fp64] [--only-split]

`value`  device-resident throughput: K steps replayed from the captured step
         graph, timed with CUDA events on the context's stream (inputs are
         larger than L2, or L2 is flushed between steps for small workloads).
`e2e`    the same metric through the C ABI with host buffers: every step
         copies x, y, z, radius, cell_type in (bmxg_set_state) and x, y, z,
         vel out (bmxg_get_state) from pinned host memory; the median of
         three host-timed windows of up to 20 calls.
`roofline` the force kernel (the dominant one) timed per launch with CUDA
         events in profiling mode, against the algorithmic bytes per
         particle-step (64 B for the FP32 sphere form, 80 B for FP64 spheres)
         and the measured HBM copy bandwidth.
`cpu_baseline` the oracle (plain-C restatement of the reference path,
         OpenMP over particles) on the host cores on a bounded sample.
Multi-GPU: replicas (each rank runs its own copy of the workload; no data-path
collective).  --impl reference times the CPU restatement of the reference
path on the host cores (the reference itself needs AMReX and MPI, absent).
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
sys.path.insert(0, ROOT)

METRIC = "DEM particle-steps/s on 1 GB300: FP64 plain vs FP32 batched @ rel force err≤1e-5"
UNIT = "particle-steps/s"
L2_BYTES = 129 * 2 ** 20
ALG_BYTES = {("sphere", 1): 64, ("sphere", 0): 80, ("rod", 1): 188, ("rod", 0): 212}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="colonies",
                    choices=["colonies", "sphere_fp32", "sphere_plain", "rod_trees"])
    ap.add_argument("--precision", default=None, choices=[None, "fp32f", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--only-main", action="store_true",
                    help="the timed steps and the roofline leg only (no other form, end-to-end, adjoint, "
                         "division or CPU legs): the run profiles capture")
    ap.add_argument("--eager", action="store_true",
                    help="with --only-main: every step launched kernel by kernel (profiling mode) from the start, "
                         "so a profiler sees the first list build as the first build launch")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="print only the differentiation form's cost on its configuration (20 000 spheres, 200 steps)")
    ap.add_argument("--only-split", action="store_true",
                    help="print only the cell-division measurements (2 731 333 records, YEAST and FUNGI)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(ms, device):
    """The slowest rank's time: every rank runs the same replica workload and
    the whole job is done when the last one is (no-op on one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def workload(name):
    from boltzmannmfx_gb300 import configs
    return {"colonies": configs.colonies, "sphere_fp32": configs.sphere_fp32,
            "sphere_plain": configs.sphere_plain, "rod_trees": configs.rod_trees}[name]()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[2 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(key):
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        v = d.get(key)
        if isinstance(v, dict):
            return v.get("bytes_per_launch")
    return None


def adjoint_cost(Context, configs, BMXG_FP64, nsteps=200, ckpt=20):
    """The differentiation form on its configuration (20 000 spheres, 200
    steps, checkpoint every 20, loss mean |x_T - target|^2, every extension
    parameter on): device time of bmxg_forward, of bmxg_backward (reverse
    sweep with checkpoint recomputation) and of the plain FP64 step, per step."""
    w = configs.adjoint_spheres()
    rng = np.random.default_rng(configs.SEED + 1)
    adh = rng.uniform(0.0, 1.0e-3, w.n)
    ctx = Context(w.params, w.geoms)
    P = w.particles
    target = np.stack([P["x"], P["y"], P["z"]]) + rng.normal(0.0, 1.0e-4, (3, w.n))

    def fwd(T):
        ctx.set_state(P)
        ctx.set_ext(0.05, 1.0e-2, adh)
        ctx.forward(w.dt, T, ckpt)
        f_ms = ctx.stats()["last_step_ms"]
        Q = P.copy()
        ctx.get_state(Q, ("x", "y", "z"))
        xT = np.stack([Q["x"], Q["y"], Q["z"]])
        return f_ms, 2.0 * (xT - target) / w.n

    _, g = fwd(ckpt)  # warm-up: compile-free, but first-touch allocations
    ctx.backward(g)
    f_ms, g = fwd(nsteps)
    ctx.backward(g)
    b_ms = ctx.stats()["last_step_ms"]
    ctx.set_state(P)
    ctx.set_ext(0.0, 0.0, None)
    ctx.step(w.dt, 8, BMXG_FP64)
    ctx.set_state(P)
    ctx.step(w.dt, nsteps, BMXG_FP64)
    p_ms = ctx.stats()["last_step_ms"]
    ctx.close()
    return {"workload": w.name, "particles": w.n, "steps": nsteps, "ckpt_every": ckpt,
            "params": "positions, stiffness, damping, drag, per-particle adhesion",
            "forward_ms_per_step": f_ms / nsteps, "adjoint_ms_per_step": b_ms / nsteps,
            "plain_fp64_ms_per_step": p_ms / nsteps,
            "adjoint_over_forward": b_ms / f_ms, "adjoint_over_plain_fp64": b_ms / p_ms,
            "bar": "adjoint <= 3x the forward step: adjoint_over_forward compares it with the forward it "
                   "differentiates (bmxg_forward, the law with every extension on); adjoint_over_plain_fp64 "
                   "with the plain FP64 step of the reference law"}


def split_cost(n, seed, reps=10, frac=0.05, fungi=False):
    """Cell division (bmxg_split_cells_aos) on n device-resident AoS records
    (BMX's 448-byte particles, seeded draws): YEAST cells with about frac of
    them above max_vol, or (fungi) hyphal segments in every state checkSplit
    looks at, about frac of them dividing.  Device time per call with CUDA
    events around it on torch's stream (each call on a fresh copy of the
    records; the call includes its host reads of the totals), the host-buffer
    call's wall time, and the oracle on the same records on one host core.
    Algorithmic bytes per call: 12 B per record for the decision (cell_type 4
    + vol 8; FUNGI segments also position, n_bnds, radius, c_length) + 1 B per
    record of decisions written and read back + 968 B per new particle (the
    mother read 444, her changed fields written 80, the daughter written
    444)."""
    import torch
    from boltzmannmfx_gb300 import runtime
    from boltzmannmfx_gb300.abi import BMXG_DEVICE, FUNGI, INT_IDX, REAL_IDX, SplitParams, aos_dtype
    from oracle import oracle as O
    sp = SplitParams(max_vol=5.0e-10, overlap=0.2, max_len=0.0035, max_rad=0.00025,
                     brnch_prob=0.05 if fungi else 0.0, split_prob=0.1, split_len=0.0030, num_reals=9,
                     num_ints=0)
    rng = np.random.default_rng(seed)
    cap = n + n // 4
    a = np.zeros(cap, aos_dtype())
    a["pos"][:n] = rng.uniform(-1.0e-3, 1.0e-3, (n, 3))
    if fungi:
        # tips (a third at the length and radius limits), segments behind a
        # tip, interior segments; frac sets the share of tips at the limits
        pos = rng.integers(0, 4, n)
        at = rng.random(n) < 3.0 * frac
        L = np.where(at, 0.0036, 0.0030)
        rad = np.where(at, 0.00026, 0.00020)
        a["idata"][:n, INT_IDX["cell_type"]] = FUNGI
        a["idata"][:n, INT_IDX["position"]] = pos
        a["idata"][:n, INT_IDX["n_bnds"]] = np.where(pos == 3, 2, 1)
        a["idata"][:n, 15] = rng.integers(1, 3, n)
        a["rdata"][:n, REAL_IDX["c_length"]] = L
        a["rdata"][:n, REAL_IDX["radius"]] = rad
        a["rdata"][:n, REAL_IDX["theta"]] = rng.uniform(0.3, np.pi - 0.3, n)
        a["rdata"][:n, REAL_IDX["phi"]] = rng.uniform(0.0, 2.0 * np.pi, n)
        a["rdata"][:n, REAL_IDX["vol"]] = np.pi * rad * rad * L
    else:
        vol = 5.0e-10 * np.where(rng.random(n) < frac, rng.uniform(1.0001, 1.9, n), rng.uniform(0.4, 1.0, n))
        r = (3.0 * vol / (4.0 * np.pi)) ** (1.0 / 3.0)
        a["rdata"][:n, REAL_IDX["vol"]] = vol
        a["rdata"][:n, REAL_IDX["radius"]] = r
        a["rdata"][:n, REAL_IDX["area"]] = 4.0 * np.pi * r * r
    a["id"][:n] = np.arange(1, n + 1)
    a["idata"][:n, INT_IDX["id"]] = a["id"][:n]
    pristine = torch.from_numpy(a.view(np.uint8)).cuda()
    work = torch.empty_like(pristine)
    st = torch.cuda.current_stream()
    times = []
    k = 0
    for it in range(reps + 3):
        work.copy_(pristine)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        k = runtime.split_cells_aos(work.data_ptr(), n, sp, seed=it, next_id=n + 1, where=BMXG_DEVICE,
                                    cap=cap, stream=st.cuda_stream)
        e1.record(st)
        e1.synchronize()
        if it >= 3:
            times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    host_s = []
    for it in range(3):
        h = a.copy()
        t0 = time.perf_counter()
        runtime.split_cells_aos(h, n, sp, seed=it, next_id=n + 1)
        host_s.append(time.perf_counter() - t0)
    # the oracle on the draws of the last timed call (seed reps + 2), so that
    # its count is the one the GPU line reports
    last_seed = reps + 2
    h = a.copy()
    t0 = time.perf_counter()
    rc, kc = O.split_cells(h, n, sp, seed=last_seed, next_id=n + 1)
    cpu_s = time.perf_counter() - t0
    alg = 14 * n + 968 * k
    peak, _ = measured_peak()
    return {"call": "bmxg_split_cells_aos (device records)", "records": n,
            "kind": "FUNGI segments" if fungi else "YEAST cells", "new_particles": k,
            "ms_per_call": ms, "records_per_s": n / (ms * 1e-3),
            "alg_bytes": alg, "achieved_gbs": alg / (ms * 1e-3) / 1e9,
            "frac_of_measured_hbm": (alg / (ms * 1e-3) / 1e9) / peak if peak else None,
            "host_records_ms": 1e3 * float(np.median(host_s)),
            "cpu_baseline": {"kind": "port", "cores": 1, "ms_per_call": 1e3 * cpu_s,
                             "records_per_s": n / cpu_s, "rc": rc, "new_particles": kc,
                             "seed": last_seed, "same_count_as_gpu": bool(kc == k)}}


def host_link(nbytes=1 << 30, reps=3):
    """Pinned host <-> device copy rate of this machine: one 1 GiB copy each way
    alone, then both directions at once on two streams (best of reps, CUDA
    events).  The end-to-end leg's copies are held against these."""
    import torch
    h1 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d1 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def h2d():
        d1.copy_(h1, non_blocking=True)

    def d2h():
        h2.copy_(d2, non_blocking=True)

    def both():
        cur = torch.cuda.current_stream()
        s1.wait_stream(cur)
        s2.wait_stream(cur)
        with torch.cuda.stream(s1):
            d1.copy_(h1, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)
        cur.wait_stream(s1)
        cur.wait_stream(s2)

    out = {}
    for name, fn, nb in (("h2d", h2d, nbytes), ("d2h", d2h, nbytes), ("both", both, 2 * nbytes)):
        best_ms = None
        for _ in range(reps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1)
            best_ms = t if best_ms is None else min(best_ms, t)
        out[name + "_gbs"] = nb / (best_ms * 1e-3) / 1e9
    del h1, h2, d1, d2
    return out


def sample_colonies(w, target):
    """Colonies of the workload whose sizes follow its colony-size mix: every
    k-th colony in order of size (stratified), k chosen so that the sample
    holds about `target` particles; all colonies when target >= the total.
    Returns (particles, geometries, offsets, colonies taken)."""
    from boltzmannmfx_gb300.abi import Particles
    sizes = np.diff(w.offsets)
    ncol = len(sizes)
    if target >= int(sizes.sum()):
        return w.particles, list(w.geoms), np.asarray(w.offsets), ncol
    order = np.argsort(sizes, kind="stable")
    k = max(1, int(round(sizes.sum() / max(target, 1))))
    # (at least one colony: a colony is the smallest unit the step runs on)
    pick = np.sort(order[min(k // 2, ncol - 1)::k])
    parts = [w.particles.subset(int(w.offsets[c]), int(w.offsets[c + 1])) for c in pick]
    P = Particles.concat(parts)
    off = np.zeros(len(pick) + 1, np.int64)
    off[1:] = np.cumsum(sizes[pick])
    return P, [w.geoms[c] for c in pick], off, len(pick)


def cpu_rate(w, nth):
    """Particle-steps/s of the oracle on one step of a ~100 000-particle
    stratified sample (calibration for the sample sizes below)."""
    from oracle import oracle as O
    P, g, off, _ = sample_colonies(w, 100_000)
    t1 = O.time_evolve(w.params, g, off, P, w.dt, 1, nth)
    return P.n / max(t1, 1e-9)


def cpu_baseline(w, budget_s=12.0):
    """Oracle (OpenMP over particles, all host threads) on a bounded sample of
    the workload: a stratified sample of colonies (the workload's colony-size
    mix) and the steps that fill ~budget_s of CPU work."""
    from oracle import oracle as O
    O.build(ref=False)
    nth = os.cpu_count() or 1
    rate = cpu_rate(w, nth)
    P, g, off, take = sample_colonies(w, min(w.n, int(rate * budget_s / 20)))
    steps = int(max(1, min(w.steps, budget_s * rate / max(P.n, 1))))
    t = O.time_evolve(w.params, g, off, P, w.dt, steps, nth)
    return {"value": P.n * steps / t, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{take} of {len(w.offsets) - 1} colonies, stratified by size ({P.n} particles, "
                      f"{100.0 * P.n / w.n:.1f} % of the workload) x {steps} steps, FP64, {t:.1f} s wall"}


def run_reference(args):
    """The CPU restatement of the reference path with all host threads, on the
    whole workload when warm-up + timed steps fit in ~150 s of CPU work, else
    on a stratified sample of its colonies that does."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = workload(args.workload)
    from oracle import oracle as O
    O.build(ref=False)
    nth = os.cpu_count() or 1
    rate = cpu_rate(w, nth)
    target = int(rate * 150.0 / max(args.steps + args.warmup, 1))
    P, g, off, take = sample_colonies(w, min(w.n, target))
    n = P.n
    O.time_evolve(w.params, g, off, P, w.dt, args.warmup, nth)
    t = O.time_evolve(w.params, g, off, P, w.dt, args.steps, nth)
    v = n * args.steps / t
    whole = n == w.n
    sample = ("the whole workload" if whole else
              f"{take} of {len(w.offsets) - 1} colonies, stratified by size ({n} particles, "
              f"{100.0 * n / w.n:.1f} % of the workload)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic, seeded (the configurations' sizes and distributions)",
            "config": {"workload": w.name, "particles": w.n, "sample_particles": n, "sample_colonies": take,
                       "sampled_fraction": n / w.n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"{sample} per step, FP64, OpenMP"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU restatement of the reference path (oracle/bmx_oracle.c); the reference "
                    "itself needs AMReX and MPI, which are not available"}
    print(json.dumps(line), flush=True)


def pinned_particles(P, fields):
    """Copy of the fields in page-locked host memory (numpy views of pinned torch tensors)."""
    import torch
    from boltzmannmfx_gb300.abi import Particles
    Q = Particles.__new__(Particles)
    Q.n, Q.rods, Q.a = P.n, P.rods, {}
    keep = []
    for k, v in P.a.items():
        if k in fields:
            t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32,
                            pin_memory=True)
            a = t.numpy()
            a[...] = v
            keep.append(t)
            Q.a[k] = a
        else:
            Q.a[k] = v
    Q._pinned = keep
    return Q


def run_ours(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from boltzmannmfx_gb300 import Context, build, configs
    from boltzmannmfx_gb300.abi import BMXG_FP32F, BMXG_FP64
    if rank == 0:
        build.build()
    if world > 1:
        dist.barrier()
    w = workload(args.workload)
    prec = {"fp32f": BMXG_FP32F, "fp64": BMXG_FP64, None: w.precision}[args.precision]
    kind = "rod" if w.particles.rods else "sphere"
    N = w.n
    stream = torch.cuda.Stream()
    ctx = Context(w.params, w.geoms)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_state(w.particles, w.offsets)
    ctx.autotune(os.path.join(ROOT, "boltzmannmfx_gb300", "_build", "autotune.json"))
    shapes = ctx.shapes()
    ctx.set_state(w.particles, w.offsets)
    state_bytes = N * (24 * 2 + 16 * 2 + 8 * 2 + 4 * 2 + 8 + 4 + 1 + 24)
    flush = state_bytes < 2 * L2_BYTES
    scratch = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda") if flush else None

    def timed_steps(precision, K):
        """K steps; device time in ms summed over CUDA-event brackets."""
        if not flush:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
            ctx.step(w.dt, K, precision)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            return e0.elapsed_time(e1)
        tot = 0.0
        for _ in range(K):
            with torch.cuda.stream(stream):
                scratch.add_(1.0)   # write a buffer larger than L2
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            ctx.step(w.dt, 1, precision)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return tot

    if args.eager and args.only_main:
        ctx.set_profiling(True)
    # the step graphs instantiated up front (bmxg_prepare: no step runs), then
    # the warm-up and the timed K steps
    ctx.prepare(w.dt, prec)
    timed_steps(prec, max(args.warmup, 3))
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    s0 = ctx.stats()
    l0, r0 = s0["n_kernel_launches"], s0["n_rebins"]
    with ClockSampler(local) as clk:
        ms = timed_steps(prec, args.steps)
    torch.cuda.synchronize()
    s1 = ctx.stats()
    launches = s1["n_kernel_launches"] - l0
    rebins = s1["n_rebins"] - r0  # bin-order rebuilds: one per step, or one per list build
    list_mode = kind == "sphere" and prec == BMXG_FP32F and rebins < args.steps
    ms = max_over_ranks(ms, "cuda")
    value = N * world * args.steps / (ms / 1e3)

    # roofline: the force kernel timed per launch (profiling mode, eager
    # launches) over the same trajectory as the timed steps: the state is
    # loaded again and stepped through the same warm-up first
    ctx.set_state(w.particles, w.offsets)
    timed_steps(prec, max(args.warmup, 3))
    ctx.set_profiling(True)
    kprof = args.steps
    timed_steps(prec, kprof)
    st = ctx.stats()
    ctx.set_profiling(False)
    k_ms = st["main_kernel_ms"] / max(st["main_kernel_launches"], 1)
    # the force error of the kernel the timed steps ran: one more step of this
    # trajectory (a list step where the list path runs) against an FP64 step
    # from the same positions (the FP64 GPU step is bit-exact to the oracle)
    Ps = w.particles.copy()
    ctx.get_state(Ps, ("x", "y", "z") + (("theta", "phi") if kind == "rod" else ()))
    r0 = ctx.stats()["n_rebins"]
    V32 = w.particles.copy()
    if prec == BMXG_FP32F:
        ctx.step(w.dt, 1, prec)
        ctx.get_state(V32, ("velx", "vely", "velz"))
    else:  # an FP64 headline: the FP32F form's step from the same positions
        c32 = Context(w.params, w.geoms)
        c32.set_state(Ps, w.offsets)
        c32.step(w.dt, 1, BMXG_FP32F)
        c32.get_state(V32, ("velx", "vely", "velz"))
        c32.close()
    step_was_list = kind == "sphere" and prec == BMXG_FP32F and ctx.stats()["n_rebins"] - r0 <= 1 and list_mode
    ref_ctx = Context(w.params, w.geoms)
    ref_ctx.set_state(Ps, w.offsets)
    ref_ctx.step(w.dt, 1, BMXG_FP64)
    V64 = w.particles.copy()
    ref_ctx.get_state(V64, ("velx", "vely", "velz"))
    ref_ctx.close()
    v32 = np.stack([V32["velx"], V32["vely"], V32["velz"]])
    v64 = np.stack([V64["velx"], V64["vely"], V64["velz"]])
    traj_err = float(np.abs(v32 - v64).max() / np.abs(v64).max())
    alg = ALG_BYTES[(kind, 1 if prec == BMXG_FP32F else 0)] * N
    peak, peak_kind = measured_peak()
    achieved = alg / (k_ms / 1e3) / 1e9
    if list_mode:
        kname = "k_list_step"
    elif kind == "rod" and prec == BMXG_FP32F:  # the events bracket the three kernels of the rod pipeline
        kname = "k_rod_pair32 + k_rod_pair64 + k_rod_seg32"
    else:
        kname = ("k_sphere" if kind == "sphere" else "k_rod_force") + ("<FP32F>" if prec == BMXG_FP32F else "<FP64>")
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind, "kernel_ms": k_ms,
            "algorithmic_bytes_per_launch": alg,
            "traffic": ncu_traffic(f"{w.name}:{kname}")}

    if args.only_main:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": ms / args.steps, "roofline": roof,
                              "gpu_launches": int(launches), "list_builds": int(rebins),
                              "launch_shapes": shapes,
                              "note": "--only-main: a profiling run, not a bench line"}), flush=True)
        ctx.close()
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    # the other form on the same workload, and the FP32F force error against FP64
    other = BMXG_FP64 if prec == BMXG_FP32F else BMXG_FP32F
    ctx.set_state(w.particles, w.offsets)
    ctx.prepare(w.dt, other)
    timed_steps(other, 3)
    ms_other = timed_steps(other, args.steps)
    v_other = N * args.steps / (ms_other / 1e3)
    fields = ("velx", "vely", "velz", "x")
    ctx.set_state(w.particles, w.offsets)
    ctx.step(w.dt, 1, BMXG_FP64)
    A = w.particles.copy()
    ctx.get_state(A, fields)
    ctx.set_state(w.particles, w.offsets)
    ctx.step(w.dt, 1, BMXG_FP32F)
    B = w.particles.copy()
    ctx.get_state(B, fields)
    va = np.stack([A["velx"], A["vely"], A["velz"]])
    vb = np.stack([B["velx"], B["vely"], B["velz"]])
    rel_err_first = float(np.abs(va - vb).max() / np.abs(va).max())

    # end to end through the C ABI with pinned host buffers
    fin = ("x", "y", "z", "radius", "cell_type")
    fout = ("x", "y", "z", "velx", "vely", "velz")
    if kind == "rod":  # segments: orientation, shape, identity and the bond table in; orientation out
        fin += ("c_length", "theta", "phi", "area", "bond_scale", "id", "cpu", "n_bnds", "seg_id1", "seg_id2",
                "site", "position", "fuse_tip", "fix_site")
        fout += ("theta", "phi", "wx", "wy", "wz", "n_bnds", "seg_id1", "seg_id2", "site", "position")
    H = pinned_particles(w.particles, set(fin) | set(fout))
    ke = min(args.steps, 20)
    for _ in range(2):
        ctx.set_state(H, w.offsets, fields=fin)
        ctx.step(w.dt, 1, prec)
        ctx.get_state(H, fout)
    # three windows of ke calls, timed on the host clock; the median window
    # is reported (one host stall in a window does not set the figure)
    wins = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ke):
            ctx.set_state(H, w.offsets, fields=fin)
            ctx.step(w.dt, 1, prec)
            ctx.get_state(H, fout)
        wins.append(time.perf_counter() - t0)
    te = float(np.median(wins))
    e2e = {"value": N * world * ke / te, "unit": UNIT,
           "h2d_bytes_per_step": int(H.nbytes(fin)), "d2h_bytes_per_step": int(H.nbytes(fout)),
           "steps": ke, "windows_ms_per_call": [round(1e3 * t / ke, 4) for t in wins],
           "path": "bmxg_set_state + bmxg_step + bmxg_get_state (host buffers)",
           "note": "a caller loading back the state it stored keeps the device's slot order and list; "
                   "the median of three windows of `steps` calls"}
    # the same calls when every load differs from the stored state (as after
    # split_particles and ParticleExchange in bmx::Evolve): one particle moved
    # by one ulp each call, so each load re-sorts and the step runs the
    # per-step path
    wins = []
    for r in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for it in range(ke):
            k = (r * ke + it) % N
            H["x"][k] = np.nextafter(H["x"][k], 1.0)
            ctx.set_state(H, w.offsets, fields=fin)
            ctx.step(w.dt, 1, prec)
            ctx.get_state(H, fout)
        wins.append(time.perf_counter() - t0)
    tc = float(np.median(wins))
    e2e_changed = {"value": N * world * ke / tc, "unit": UNIT, "steps": ke, "ms_per_call": 1e3 * tc / ke,
                   "windows_ms_per_call": [round(1e3 * t / ke, 4) for t in wins],
                   "path": "the e2e calls with a changed state every call (full load); the median of three windows"}

    adj = None
    split = None
    if rank == 0 and w.name.startswith("colonies"):
        adj = adjoint_cost(Context, configs, BMXG_FP64)
        split = [split_cost(N, configs.SEED + 2), split_cost(N, configs.SEED + 3, fungi=True)]

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(w)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if prec == BMXG_FP32F else "f64",
                "data": "synthetic, seeded (the configurations' sizes and distributions)",
                "config": {"workload": w.name, "particles": N, "colonies": w.ncol,
                           "form": "FP32F" if prec == BMXG_FP32F else "FP64",
                           "parallelism": f"replicas x{world}",
                           "l2": ("L2 flushed between steps" if flush else
                                  f"inputs larger than L2 (state {state_bytes / 2**20:.0f} MiB)")},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "adjoint": adj, "split": split,
                "step_structure": ({"kind": "FP32F neighbour list with a skin", "list_builds": int(rebins),
                                    "steps": args.steps,
                                    "per_step": "k_list_decide + k_list_step",
                                    "per_build": "k_list_rebin, 3 scan kernels, k_list_scatter, k_list_canon, "
                                                 "k_list_cells, k_list_build, 3 scan kernels, "
                                                 "k_list_xcopy "
                                                 "(CUDA-graph conditional node)"}
                                   if list_mode else
                                   {"kind": "per-step binning", "rebins": int(rebins), "steps": args.steps}),
                "clocks": clk.summary(),
                "launch_shapes": dict(shapes, source="bmxg_autotune (cache keyed by device, n, colony-size "
                                                     "histogram)"),
                "other_form": {"form": "FP64" if other == BMXG_FP64 else "FP32F", "value": v_other,
                               "unit": UNIT, "ms_per_step": ms_other / args.steps},
                "fp32f_over_fp64": (value / v_other) if prec == BMXG_FP32F else (v_other / value),
                "rel_force_err_fp32f_vs_fp64": traj_err,
                "force_err": {"kernel": ("k_list_step" if step_was_list else
                                         kname if prec == BMXG_FP32F else
                                         ("k_sphere<FP32F>" if kind == "sphere" else "FP32F rod pipeline")),
                              "how": "one more FP32F step at the end of the roofline leg's trajectory against an "
                                     "FP64 step from the same positions (an FP64 headline: the FP32F step from "
                                     "its positions); max-norm relative velocity error",
                              "value": traj_err,
                              "first_step_after_load": {"kernel": "k_sphere<FP32F>" if kind == "sphere" else kname,
                                                        "value": rel_err_first}},
                "host_link": host_link(),
                "e2e_changed_state": e2e_changed}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.only_adjoint:
        import torch
        from boltzmannmfx_gb300 import Context, build, configs
        from boltzmannmfx_gb300.abi import BMXG_FP64
        build.build()
        torch.cuda.set_device(0)
        print(json.dumps(adjoint_cost(Context, configs, BMXG_FP64)), flush=True)
    elif args.only_split:
        from boltzmannmfx_gb300 import build, configs
        build.build()
        print(json.dumps(split_cost(2731333, configs.SEED + 2)), flush=True)
        print(json.dumps(split_cost(2731333, configs.SEED + 3, fungi=True)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
