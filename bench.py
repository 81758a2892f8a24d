"""Benchmark: tracer-cell updates/s of 3-D LOBSTER with carbonates on one GB300.

Workload: 256 x 256 x 64 grid (50 km x 50 km x 500 m, Periodic/Periodic/Bounded), 11 advected tracers
(NO3 NH4 P Z sPOM bPOM DOM DIC Alk + T S), seeded initial conditions, a divergence-free velocity
from a seeded random streamfunction (0.1 m/s RMS), TwoBand PAR with the default surface PAR,
WENO5 advection + sinking + LOBSTER + RK3, dt = 300 s.  One tracer-cell update = one tracer
advanced one full RK3 step (three substeps) in one cell.

Arms:
  default           the fused CUDA path through the C ABI (state resident in HBM for `value`;
                    `e2e` copies the whole state host->device and back around every step, with
                    two ensemble members alternating so that one's copies overlap the other's step).
  --impl reference  the CPU restatement of the reference's path (the reference itself is Julia and
                    cannot run here), all host cores, on a bounded sample of the same workload.
Multi-GPU: each rank runs an independent replica (weak scaling, no data-path collective).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oceanbiome.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

SHAPE = (256, 256, 64)
EXTENT = (50_000.0, 50_000.0, 500.0)
DT = 300.0
N_TRACERS = 11
E2E_MEMBERS = 4
METRIC = "tracer-cell updates/s"
WORKLOAD = "LOBSTER+carbonates 3-D, 256x256x64, 11 tracers, WENO5 + sinking + TwoBand PAR + RK3, dt=300 s"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp64_peak():
    """Measured FP64 FMA rate of this GPU (GFLOP/s) from the library's probe kernel."""
    import ctypes as C
    from obgc import _abi as A
    x = C.c_double()
    A.check(A.load().obgc_fp64_fma_peak(C.byref(x), None), "obgc_fp64_fma_peak")
    return x.value


# FP64 FLOPs per cell (2 per DFMA + DMUL + DADD) from ncu's sass counters of one launch on these
# workloads: the pH solve from a cold start (~5 Newton iterations) and PISCES' warm-started Omega,
# both with the default TEOS-10 polynomial density
CARBON_FLOP_PER_CELL = 1671.0
OMEGA_FLOP_PER_CELL = 1529.0


def e2e_members_ms(members, nsteps, stream, lanes=2, trials=1, info=None):
    """End-to-end steps of an ensemble through the public API, the way a host drives several model
    members on one GPU: member k % M takes step k, which copies that member's fields in from pinned
    host memory (copy-in streams), steps it on the launching stream and reads its result back
    (read-back streams).  A member's copy-in waits for its previous read-back, and its step for its
    copy-in, so every step still moves its whole state both ways; the copies of one member overlap
    the step of another.  Each direction spreads its fields over `lanes` streams.  One untimed
    round of copies both ways comes first: on GB300 the first copies from freshly pinned buffers ran
    at about 90 GB/s, later ones at about 205 GB/s host to device and 189 GB/s back (156 GB/s each
    way when both directions run at once).  members: [(step, dev fields, pinned host fields)].  Returns ms per step (CUDA events on the launching stream, which joins every copy
    stream before the end event): the median of `trials` timed runs of nsteps steps.  info (a dict,
    optional) receives every trial's ms per step and the host link's rates in the untimed round
    (GB/s, each direction alone), since the pipeline is bound by that link when the machine's other
    work loads it."""
    import torch
    M = len(members)
    ins = [torch.cuda.Stream() for _ in range(lanes)]
    outs = [torch.cuda.Stream() for _ in range(lanes)]
    copied = [[torch.cuda.Event() for _ in range(lanes)] for _ in range(M)]
    stepped = [torch.cuda.Event() for _ in range(M)]
    read = [[torch.cuda.Event() for _ in range(lanes)] for _ in range(M)]
    # untimed: both directions once, each direction timed alone
    c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    nbytes = sum(h.numel() * h.element_size() for _, _, host in members for h in host.values())
    torch.cuda.synchronize()
    c0.record(stream)
    with torch.cuda.stream(stream):
        for _, dev, host in members:
            for n in dev:
                dev[n].copy_(host[n], non_blocking=True)
        c1.record(stream)
        for _, dev, host in members:
            for n in dev:
                host[n].copy_(dev[n], non_blocking=True)
        c2.record(stream)
    torch.cuda.synchronize()
    if info is not None:
        info["host_link_gbs"] = {"h2d": nbytes / c0.elapsed_time(c1) / 1e6, "d2h": nbytes / c1.elapsed_time(c2) / 1e6}
    runs = sorted(_e2e_trial(members, nsteps, stream, ins, outs, copied, stepped, read) for _ in range(trials))
    if info is not None:
        info["trials_ms_per_step"] = runs
    return runs[len(runs) // 2]


def _e2e_trial(members, nsteps, stream, ins, outs, copied, stepped, read):
    import torch
    M, lanes = len(members), len(ins)
    start = torch.cuda.Event()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    start.record(stream)
    for s in ins + outs:
        s.wait_event(start)
    for k in range(nsteps):
        m = k % M
        step, dev, host = members[m]
        names = list(dev)
        for q, s in enumerate(ins):
            if k >= M:
                for ev in read[m]:
                    s.wait_event(ev)
            with torch.cuda.stream(s):
                for n in names[q::lanes]:
                    dev[n].copy_(host[n], non_blocking=True)
                copied[m][q].record(s)
        for ev in copied[m]:
            stream.wait_event(ev)
        step()
        stepped[m].record(stream)
        for q, s in enumerate(outs):
            s.wait_event(stepped[m])
            with torch.cuda.stream(s):
                for n in names[q::lanes]:
                    host[n].copy_(dev[n], non_blocking=True)
                read[m][q].record(s)
    for m in range(min(M, nsteps)):
        for ev in read[m]:
            stream.wait_event(ev)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / nsteps


def algorithmic_bytes_per_update(state_bytes, g_bytes, vel_bytes, n_tracers, n_vel):
    """Per tracer-cell update (3 substeps): U read x3 + U write x3 (state precision), G write x2 +
    G- read x2 (tendency precision), and n_vel velocity components read x3 shared by all tracers."""
    return 6 * state_bytes + 4 * g_bytes + 3 * n_vel * vel_bytes / n_tracers


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(steps=None, threads=None, warmup=1, seconds=10.0):
    """The oracle (CPU restatement of the reference's path) on the workload's own 256 x 256 x 64
    grid with the GPU arm's seeds, FP64, all host threads: `warmup` untimed steps, then `steps`
    timed steps (default: as many as fit about `seconds`, at most 30)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import obgc
    threads = threads or (os.cpu_count() or 1)
    shape = SHAPE
    g = obgc.RectilinearGrid(shape, EXTENT)
    p = O.preset("LOBSTER")
    p.carbonate_system = 1
    names = ["NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM", "DIC", "Alk", "T", "S"]
    m = O.model3d(p, g.c_grid(), names)
    init = obgc.lobster_initial_conditions(g, seed=11)   # the GPU arm's seeds (rank 0)
    st = np.ascontiguousarray(np.stack([np.broadcast_to(np.asarray(init[n], dtype=np.float64), g.shape) for n in names]))
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=7, device="cpu")
    u = u.numpy().ravel().copy()
    v = v.numpy().ravel().copy()
    t = 0.0
    one = None
    for _ in range(max(1, warmup)):
        t0 = time.perf_counter()
        O.step3d(m, st, u=u, v=v, t=t, dt=DT, nsteps=1, threads=threads)
        one = time.perf_counter() - t0
        t += DT
    if steps is None:
        steps = max(1, min(30, int(seconds / max(one, 1e-3))))
    t0 = time.perf_counter()
    O.step3d(m, st, u=u, v=v, t=t, dt=DT, nsteps=steps, threads=threads)
    el = time.perf_counter() - t0
    value = N_TRACERS * g.N * steps / el
    return {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} RK3 steps of the 256x256x64 LOBSTER+carbonates grid (11 tracers), FP64, "
                      f"{el:.1f} s"}, el / steps


def precision_arm(prec, steps, shape=SHAPE, rank=0):
    """Tracer-cell updates/s of the same workload at another precision (state resident in HBM,
    CUDA events around `steps` steps after two warm-up steps)."""
    import torch
    import obgc
    extent = (EXTENT[0] * shape[0] / SHAPE[0], EXTENT[1] * shape[1] / SHAPE[1], EXTENT[2])
    g = obgc.RectilinearGrid(shape, extent, ("Periodic", "Periodic", "Bounded"), dtype="f32" if prec == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=7 + rank)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision=prec)
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=11 + rank))
    obgc.time_step(model, DT, nsteps=2)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    obgc.time_step(model, DT, nsteps=steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"value": N_TRACERS * g.N / (ms / 1e3), "unit": METRIC, "ms_per_step": ms, "steps": steps,
            "dtype": {"f32": "f32", "mixed": "f64-state/f32-compute", "f64": "f64"}[prec]}


def timed_precision_error(prec, steps=1000, shape=(32, 32, 16)):
    """The error statement of a precision after `steps` steps of the workload's physics on a small
    grid, against the FP64 oracle on the host, with the oracle's envelope for FP32 rounding (one
    seeded rounding per stored value and stage) and for FP64 rounding beside it."""
    import numpy as np
    import torch
    import obgc
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import conditioning as K
    t0 = time.perf_counter()
    c = K.LobsterCase(shape)
    ref = c.oracle_run(steps)
    ph_ref = K.ph_total(ref)
    g = obgc.RectilinearGrid(c.shape, c.extent, ("Periodic", "Periodic", "Bounded"), dtype="f32" if prec == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=c.vel_seed)
    m = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision=prec)
    obgc.set_(m, **c.init)
    obgc.time_step(m, DT, nsteps=steps, graph=True)
    torch.cuda.synchronize()
    got = m.state_array().cpu().numpy().astype(np.float64)
    stmt = K.error_statement(got, ref)
    return {"precision": prec, "steps": steps, "grid": list(shape), "dt_s": DT,
            "against": "FP64 oracle on the host, same inputs",
            "worst": K.summary(stmt, K.ph_total(got), ph_ref),
            "tracers": {n: {k: float("%.3g" % x) for k, x in e.items()} for n, e in stmt.items()},
            "oracle_envelope_f32_rounding": c.envelope(ref, ph_ref, steps, K.U32, seeds=(1,)),
            "oracle_envelope_f64_rounding": c.envelope(ref, ph_ref, steps, K.U64, seeds=(1,)),
            "bounds": {"tracer_rel": 1e-5, "pH_abs": 1e-8},
            "note": "cellwise bounds lie below the oracle's own FP64-rounding envelope; the normwise 1e-5 is met",
            "seconds": time.perf_counter() - t0}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    # the full 256 x 256 x 64 workload: W untimed warm-up steps, then K timed steps
    base, per_step = cpu_baseline(steps=args.steps, warmup=args.warmup)
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded LOBSTER initial conditions and "
                                                        "random-streamfunction velocity)",
            "config": {"workload": WORKLOAD, "grid": list(SHAPE), "tracers": N_TRACERS, "dt_s": DT,
                       "precision": "f64", "sample": base["sample"], "parallelism": "host threads"},
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    import obgc
    from obgc import _abi as A
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    lib = A.load()

    prec = args.precision
    shape = tuple(args.shape) if args.shape else SHAPE
    extent = (EXTENT[0] * shape[0] / SHAPE[0], EXTENT[1] * shape[1] / SHAPE[1], EXTENT[2])
    g = obgc.RectilinearGrid(shape, extent, ("Periodic", "Periodic", "Bounded"), dtype="f32" if prec == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=7 + rank)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=prec)
    if args.tz:
        model.set_tiling(args.tz)
    if args.staging != "default":
        model.set_staging(1 if args.staging == "tma" else 0)
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=11 + rank))
    assert len(model.tracer_names) == N_TRACERS
    # the launch shape: the library's autotuner on this state (restored afterwards), outside the
    # timed region, unless the command line fixes the shape
    tuning = {"levels_per_item": args.tz or "rule", "staging": args.staging, "autotuned": False}
    if not args.tz and args.staging == "default" and not args.no_autotune:
        tz, sg, tms = model.autotune(DT, steps=3)
        tuning = {"levels_per_item": tz, "staging": "tma" if sg else "cp.async", "autotuned": True,
                  "autotune_ms_per_step": tms}

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up (also builds the CUDA graph)
    obgc.time_step(model, DT, nsteps=max(args.warmup, 3) if args.warmup > 0 else 3, graph=True)
    barrier()

    # ---- value: state resident in HBM, K steps in one graph replay per call, profiled launches
    model.set_profiling(True)
    launches0 = lib.obgc_kernel_launch_count()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        ev0.record(stream)
        obgc.time_step(model, DT, nsteps=args.steps)
        ev1.record(stream)
        barrier()
    launches = lib.obgc_kernel_launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    _, substep_ms, _ = model.last_timing()
    staging = "tma" if model.staging()[1] else "cp.async"
    model.set_profiling(False)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = t.item()
    updates = N_TRACERS * g.N * args.steps * world
    value = updates / (ms / 1e3)

    # ---- e2e: public API with host buffers: every step copies a member's whole state in from
    # pinned host memory, steps it and copies it back; E2E_MEMBERS ensemble members (model contexts)
    # take the steps in turn, so that a member's read-back and next copy-in overlap the other members'
    # steps (with two members the copies of one member, 2 x 185 MB, outlast the other's step)
    names = model.tracer_names
    others = []
    for q in range(E2E_MEMBERS - 1):
        mq = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                      precision=prec)
        if args.tz or tuning["autotuned"]:
            mq.set_tiling(tuning["levels_per_item"])
        if args.staging != "default" or tuning["autotuned"]:
            mq.set_staging(1 if tuning["staging"] == "tma" else 0)
        obgc.set_(mq, **obgc.lobster_initial_conditions(g, seed=23 + 7 * q + rank))
        obgc.time_step(mq, DT, nsteps=1, graph=True)          # warm-up: builds its graph
        others.append(mq)
    members = []
    for mdl in [model] + others:
        host = {n: torch.empty(g.shape, dtype=mdl.state_dtype, pin_memory=True) for n in names}
        for n in names:
            host[n].copy_(mdl.tracers[n])
        members.append(((lambda mdl=mdl: obgc.time_step(mdl, DT, nsteps=1, graph=True)),
                        {n: mdl.tracers[n] for n in names}, host))
    barrier()
    e2e_steps = max(2 * E2E_MEMBERS, min(args.steps, 200))   # the value leg's K steps
    h2d = sum(h.numel() * h.element_size() for h in members[0][2].values())
    e2e_info = {}
    e2e_ms = e2e_members_ms(members, e2e_steps, stream, trials=3, info=e2e_info)
    barrier()
    e2e_value = N_TRACERS * g.N * world / (e2e_ms / 1e3)
    del others, members

    # ---- roofline of the fused substep kernel
    s = 4 if prec == "f32" else 8
    gb = 4 if prec != "f64" else 8
    bytes_per_update = algorithmic_bytes_per_update(s, gb, s, N_TRACERS, 2)
    substep_avg_ms = substep_ms / (3 * args.steps) if substep_ms > 0 else ms / (3 * args.steps)
    bytes_per_launch = bytes_per_update * N_TRACERS * g.N / 3
    achieved = bytes_per_launch / (substep_avg_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    # DRAM bytes per cell of one substep launch, FP32: dram__bytes_read.sum + dram__bytes_write.sum of
    # the ncu capture of an RK3 stage-2 launch (TMA-staged) at 256x256x32 (372.9 MB / 2,097,152
    # cells), scaled by the cells of this grid
    traffic = 177.8 * g.N if prec == "f32" else None

    # the other precisions of the same workload (the metric's mixed vs FP64), and the error
    # statement of the timed precision after 1000 steps against the FP64 oracle
    arms, err = None, None
    if rank == 0 and not args.no_cpu_baseline:
        arms = {p: precision_arm(p, 4 if p == "f64" else 20, shape) for p in ("f32", "mixed", "f64") if p != prec}
        arms[prec] = {"value": value, "unit": METRIC, "ms_per_step": ms / args.steps, "steps": args.steps}
        f64v = arms["f64"]["value"]
        for p in arms:
            arms[p]["vs_f64"] = arms[p]["value"] / f64v
        err = timed_precision_error(prec)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, _ = cpu_baseline()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"f32": "f32", "mixed": "f64-state/f32-compute", "f64": "f64"}[prec],
            "data": "synthetic (seeded LOBSTER initial conditions and random-streamfunction velocity)",
            "config": {"workload": WORKLOAD if shape == SHAPE else WORKLOAD.replace("256x256x64", "x".join(map(str, shape))),
                       "grid": list(shape), "tracers": N_TRACERS, "dt_s": DT,
                       "precision": prec, "l2": "state (%.0f MB) larger than L2 (129 MB)" % (N_TRACERS * g.N * s / 1e6),
                       "tile_staging": staging, "launch_shape": tuning,
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "ms_per_step": e2e_ms, "steps": e2e_steps,
                    "pipeline": f"{E2E_MEMBERS} ensemble members take the steps in turn: each step copies its member's "
                                "state in from pinned host memory and back; a member's copies overlap the other members' steps",
                    "trials_ms_per_step": e2e_info.get("trials_ms_per_step"), "statistic": "median of 3 trials",
                    "host_link_gbs": e2e_info.get("host_link_gbs")},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "substep_kernel", "algorithmic_bytes_per_launch": bytes_per_launch,
                         "traffic_launch": "RK3 stage 2 of 3 (U and G- read, U and G written: 184 B per cell "
                                           "algorithmic); achieved and algorithmic bytes are the 3-stage average",
                         "avg_launch_ms": substep_avg_ms},
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
            "precision_arms": arms,
            "error_statement": err,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ----------------------------------------------------------------------------- batched columns
COL_N, COL_STEPS, COL_DT = 4096, 1440, 600.0
COL_WORKLOAD = ("4096 uneven NPZD columns, 16-256 levels at 2 m, per-column growth rate / mixed layer / surface PAR, "
                "kappa 1e-4..1e-2 m2/s implicit, dt=600 s, 1440 steps")


def columns_cpu_baseline(cols, threads=None, steps=20):
    """The oracle's column runner on the first 512 columns for `steps` steps, all host threads."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import obgc
    threads = threads or (os.cpu_count() or 1)
    bgc = obgc.NPZD(None)
    names = obgc.required_biogeochemical_tracers(bgc)
    sample = cols[:512]
    so, ko, st, kp, specs = [], [], [], [], []
    a = b = 0
    for c in sample:
        Nz = c["init"].shape[1]
        so.append(a); ko.append(b)
        st.append(c["init"].ravel()); kp.append(c["kappa"])
        a += len(names) * Nz; b += Nz + 1
        specs.append(O.Column(Nz, steps, c["dz"], c["surface_PAR"], c["mu0"], c["dt"], -1, -1, 0.0))
    state = np.ascontiguousarray(np.concatenate(st))
    kappa = np.ascontiguousarray(np.concatenate(kp))
    t0 = time.perf_counter()
    O.columns_run(bgc.params, obgc._abi.default_twoband(), specs, names, state, kappa, so, ko, 0.0, 0, threads=threads)
    el = time.perf_counter() - t0
    cells = sum(c["init"].shape[1] for c in sample)
    return {"value": len(names) * cells * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(sample)} of the columns ({cells} cells) for {steps} steps, FP64, {el:.1f} s"}


def run_columns(args):
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    torch.cuda.set_device(0)
    lib = A.load()
    prec = args.precision
    steps = args.steps if args.steps_given else COL_STEPS
    warm = max(args.warmup, 3)
    cols = obgc.npzd_column_ensemble(COL_N, seed=2024, levels=(16, 256), dt=COL_DT, nsteps=10 ** 7)
    cells = sum(c["init"].shape[1] for c in cols)
    bgc = obgc.NPZD(None)
    nt = 5
    updates = nt * cells * steps

    # e2e through the public API: host columns in, `steps` steps, host results out
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng = obgc.ColumnEngine(bgc, precision=prec, max_columns=COL_N, arena_cells=cells + COL_N)
    slots = [eng.add(c["init"], c["kappa"], c["dz"], c["dt"], c["nsteps"], surface_PAR=c["surface_PAR"], mu0=c["mu0"])
             for c in cols]
    t_add = time.perf_counter() - t0
    threads, cap = eng.autotune(steps=8)
    eng.run(warm, steps_per_launch=warm, graph=False)
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    modes = {}
    launches_by_mode = {}
    with ClockSampler(0) as clocks:
        for name, K, graph in (("graph_one_launch_per_step", 1, True), ("chunk_32_steps", 32, True),
                               ("persistent_one_launch", steps, False)):
            if graph:
                eng.run(steps, steps_per_launch=K, graph=True)      # capture outside the timed region
            torch.cuda.synchronize()
            l0 = lib.obgc_kernel_launch_count()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.run(steps, steps_per_launch=K, graph=graph, stream=stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            modes[name] = {"ms": e0.elapsed_time(e1), "steps_per_launch": K, "graph": graph}
            launches_by_mode[name] = lib.obgc_kernel_launch_count() - l0
    best = min(modes, key=lambda m: modes[m]["ms"])
    ms = modes[best]["ms"]
    value = updates / (ms / 1e3)
    for m in modes.values():
        m["value"] = updates / (m["ms"] / 1e3)

    # read everything back (end of the e2e region: add + steps + read)
    t1 = time.perf_counter()
    eng.run(steps, steps_per_launch=steps, graph=False)
    outs = [eng.read(s) for s in slots]
    torch.cuda.synchronize()
    t_run_read = time.perf_counter() - t1
    assert all(np.all(np.isfinite(o)) for o in outs[:64])
    e2e_s = t_add + t_run_read
    h2d = sum(c["init"].size * 8 + c["kappa"].size * 8 for c in cols)
    d2h = sum(o.size * 8 for o in outs)
    eng.close()

    # roofline of the one-launch-per-step form (state in and out of HBM every launch)
    es = 4 if prec == "f32" else 8
    per_launch_bytes = cells * nt * es * 2 + (cells + COL_N) * es
    g = modes["graph_one_launch_per_step"]
    g_launch_ms = g["ms"] / steps
    peak, peak_kind = peaks()
    achieved = per_launch_bytes / (g_launch_ms / 1e3) / 1e9

    # plain per-run FP64 path: each column alone, all its steps in one launch, runs one after another
    sample = cols[:: COL_N // 32]
    plain_updates = 0
    plain_ms = 0.0
    for c in sample:
        e1_ = obgc.ColumnEngine(bgc, precision="f64", max_columns=1, arena_cells=c["init"].shape[1] + 1)
        e1_.add(c["init"], c["kappa"], c["dz"], c["dt"], c["nsteps"], surface_PAR=c["surface_PAR"], mu0=c["mu0"])
        e1_.run(4, steps_per_launch=4, graph=False)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        e1_.run(200, steps_per_launch=200, graph=False, stream=stream.cuda_stream)
        a1.record(stream)
        torch.cuda.synchronize()
        plain_ms += a0.elapsed_time(a1)
        plain_updates += nt * c["init"].shape[1] * 200
        e1_.close()
    plain_value = plain_updates / (plain_ms / 1e3)

    cpu = None if args.no_cpu_baseline else columns_cpu_baseline(cols)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": steps, "warmup": warm,
        "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"f32": "f32", "mixed": "f64-state/f32-compute", "f64": "f64"}[prec],
        "data": "synthetic (seeded column ensemble)",
        "config": {"workload": COL_WORKLOAD, "columns": COL_N, "cells": cells, "tracers": nt, "precision": prec,
                   "autotuned": {"threads": threads, "pack_cells": cap}, "best_mode": best, "modes": modes,
                   "l2": "state %.1f MB: packs stay in shared memory within a launch" % (cells * nt * es / 1e6)},
        "e2e": {"value": updates / e2e_s, "unit": METRIC, "h2d_bytes_per_step": h2d / steps,
                "d2h_bytes_per_step": d2h / steps, "seconds": e2e_s,
                "note": "add every column from host, run the steps, read every column back"},
        "gpu_launches": int(launches_by_mode[best]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": peak_kind, "kernel": "column_kernel (one launch per step)",
                     "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_ms": g_launch_ms,
                     "note": "the persistent and chunked forms keep each pack in shared memory across steps; "
                             "their bound is on-chip issue, not HBM"},
        "plain_fp64_per_run": {"value": plain_value, "unit": METRIC, "sample": f"{len(sample)} columns x 200 steps",
                               "speedup": value / plain_value},
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- column service
SVC_WORKLOAD = ("column-run service: LOBSTER+carbonates columns, 8-512 levels (log-uniform), 1-30 days, dt 300-1800 s, "
                "alkalinity pulse 0-500 at a random level and step, air-sea CO2 exchange on DIC (surface T 2-28 degC, "
                "S 33-37, wind 7 m/s); Poisson arrivals")
SVC_WIND = 7.0


def run_service(args):
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    torch.cuda.set_device(0)
    lib = A.load()
    prec = args.precision
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())
    co2 = obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=SVC_WIND)
    rates = args.rates or [10.0, 100.0, 1000.0]
    rng = np.random.default_rng(99)
    sweep = []
    l_total = 0
    with ClockSampler(0) as clocks:
        for lam in rates:
            n = int(min(2000, max(40, lam * args.arrival_seconds)))
            reqs = [obgc.lobster_column_request(rng) for _ in range(n)]
            gaps = rng.exponential(1.0 / lam, size=n)
            svc = obgc.ColumnService(bgc, precision=prec, max_columns=8192, arena_cells=4 << 20,
                                     chunk_steps=args.chunk, co2_exchange=co2)
            l0 = lib.obgc_kernel_launch_count()
            t = time.perf_counter()
            for r, gap in zip(reqs, gaps):
                t += gap
                while True:
                    d = t - time.perf_counter()
                    if d <= 0:
                        break
                    time.sleep(min(d, 0.002))
                svc.submit_request(r)
            svc.drain(timeout=600)
            st = svc.stats()
            svc.close()
            l_total += lib.obgc_kernel_launch_count() - l0
            col_steps = sum(r["nsteps"] * r["init"].shape[1] for r in reqs)
            sweep.append({"rate_per_s": lam, "requests": n, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                          "max_ms": st["max_ms"], "runs_per_s": n / st["span_s"] if st["span_s"] > 0 else None,
                          "tracer_cell_updates_per_s": 9 * col_steps / st["span_s"] if st["span_s"] > 0 else None,
                          "launches": st["launches"], "_reqs": reqs, "_gaps": gaps})

    # one-run-per-launch FP64: measured per-step cost by level count, then the same arrivals FCFS
    levels = [8, 32, 128, 512]
    cost = []
    stream = torch.cuda.current_stream()
    for Nz in levels:
        r = obgc.lobster_column_request(np.random.default_rng(Nz), levels=(Nz, Nz), days=(1, 1))
        e1_ = obgc.ColumnEngine(bgc, precision="f64", max_columns=1, arena_cells=Nz + 1, co2_exchange=co2)
        e1_.add(r["init"], r["kappa"], r["dz"], r["dt"], 10 ** 6, surface_PAR=r["surface_PAR"], T=r["T"], S=r["S"])
        e1_.run(4, steps_per_launch=4, graph=False)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        e1_.run(300, steps_per_launch=300, graph=False, stream=stream.cuda_stream)
        a1.record(stream)
        torch.cuda.synchronize()
        cost.append(a0.elapsed_time(a1) / 300)
        e1_.close()
    for row in sweep:
        reqs, gaps = row.pop("_reqs"), row.pop("_gaps")
        arrive = np.cumsum(gaps)
        svc_ms = np.array([np.interp(r["init"].shape[1], levels, cost) * r["nsteps"] for r in reqs])
        free, lat = 0.0, []
        for a, s_ms in zip(arrive, svc_ms):
            start = max(a, free)
            free = start + s_ms / 1e3
            lat.append((free - a) * 1e3)
        lat = np.sort(np.array(lat))
        row["baseline_fp64_one_run_per_launch"] = {
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "runs_per_s": len(reqs) / (free - arrive[0]) if free > arrive[0] else None}
    top = sweep[-1]
    line = {
        "metric": "column-run p50/p99 latency and runs/s", "value": top["runs_per_s"], "unit": "runs/s",
        "n_gpus": 1, "steps": len(rates), "warmup": 0, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"f32": "f32", "mixed": "f64-state/f32-compute", "f64": "f64"}[prec],
        "data": "synthetic (seeded requests, Poisson arrivals)",
        "config": {"workload": SVC_WORKLOAD, "precision": prec, "chunk_steps": args.chunk, "rates": rates,
                   "baseline_cost_ms_per_step_by_levels": dict(zip(map(str, levels), cost))},
        "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"], "sweep": sweep,
        "e2e": {"value": top["runs_per_s"], "unit": "runs/s", "note": "host requests in, host results out",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
        "gpu_launches": int(l_total),
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- accuracy after 1000 steps
def error_statement(got, ref, names):
    """Per tracer max |x - x_ref| and max |x - x_ref| / max(|x_ref|, 1e-6 max|x_ref|)."""
    import numpy as np
    out = {}
    for q, n in enumerate(names):
        g, r = got[q].astype(np.float64), ref[q].astype(np.float64)
        d = np.abs(g - r)
        floor = 1e-6 * max(float(np.max(np.abs(r))), 1e-300)
        out[n] = {"max_abs": float(d.max()), "max_rel": float(np.max(d / np.maximum(np.abs(r), floor)))}
    return out


def run_accuracy(args):
    """FP32 and mixed (FP64 state, FP32 compute) LOBSTER+carbonates after `steps` steps against the
    FP64 oracle (small grid, CPU) and against the FP64 GPU path (full grid), tracers and FP64 pH."""
    import numpy as np
    import torch
    import obgc
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    torch.cuda.set_device(0)
    steps = args.steps if args.steps_given else 1000
    cc = obgc.CarbonChemistry()

    def run(shape, prec, seed=3):
        extent = (EXTENT[0] * shape[0] / SHAPE[0], EXTENT[1] * shape[1] / SHAPE[1], EXTENT[2])
        g = obgc.RectilinearGrid(shape, extent, ("Periodic", "Periodic", "Bounded"),
                                 dtype="f32" if prec == "f32" else "f64")
        bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
        u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed)
        m = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=prec)
        obgc.set_(m, **obgc.lobster_initial_conditions(g, seed=seed + 1))
        s0 = m.state_array().cpu().numpy().astype(np.float64)
        obgc.time_step(m, DT, nsteps=steps, graph=True)
        torch.cuda.synchronize()
        return g, bgc, (u, v), m.tracer_names, s0, m.state_array().cpu().numpy().astype(np.float64)

    def ph(state, names):
        t = {n: torch.as_tensor(state[names.index(n)], device="cuda") for n in ("DIC", "Alk", "T", "S")}
        return cc(t["DIC"], t["T"], t["S"], Alk=t["Alk"], output="pHt").cpu().numpy()

    result = {}
    # small grid against the oracle
    small = (64, 64, 32)
    g, bgc, (u, v), names, s0, f64 = run(small, "f64")
    ref = np.ascontiguousarray(s0)
    m = O.model3d(bgc.params, g.c_grid(), names)
    t0 = time.perf_counter()
    O.step3d(m, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
             t=0.0, dt=DT, nsteps=steps, threads=os.cpu_count())
    t_oracle = time.perf_counter() - t0
    ph_ref = ph(ref, names)
    for prec, state in (("f64", f64), ("mixed", run(small, "mixed")[5]), ("f32", run(small, "f32")[5])):
        result[f"{prec}_vs_oracle_64x64x32"] = {"tracers": error_statement(state, ref, names),
                                               "pH_max_abs": float(np.max(np.abs(ph(state, names) - ph_ref)))}
    # full grid against the FP64 GPU path
    _, _, _, names, _, f64 = run(SHAPE, "f64")
    ph64 = ph(f64, names)
    for prec in ("mixed", "f32"):
        state = run(SHAPE, prec)[5]
        result[f"{prec}_vs_gpu_f64_256x256x64"] = {"tracers": error_statement(state, f64, names),
                                                  "pH_max_abs": float(np.max(np.abs(ph(state, names) - ph64)))}
    worst = {k: max(v2["max_rel"] for v2 in v["tracers"].values()) for k, v in result.items()}
    print(json.dumps({"workload": "accuracy", "steps": steps, "dt_s": DT, "oracle_seconds": t_oracle,
                      "worst_max_rel": worst, "pH_max_abs": {k: v["pH_max_abs"] for k, v in result.items()},
                      "detail": result}))
    return 0


# ----------------------------------------------------------------------------- carbonate chemistry
def run_carbon(args):
    """pH (total scale) of every cell of the 256x256x64 LOBSTER state, FP64 Newton per cell."""
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    torch.cuda.set_device(0)
    lib = A.load()
    shape = tuple(args.shape) if args.shape else SHAPE
    g = obgc.RectilinearGrid(shape, (EXTENT[0] * shape[0] / SHAPE[0], EXTENT[1] * shape[1] / SHAPE[1], EXTENT[2]))
    init = obgc.lobster_initial_conditions(g, seed=11)
    dev = {n: torch.as_tensor(np.broadcast_to(np.asarray(init[n], dtype=np.float64), g.shape).copy(),
                              device="cuda").contiguous() for n in ("DIC", "Alk", "T", "S")}
    cc = obgc.CarbonChemistry()
    n = g.N
    for _ in range(max(args.warmup, 3)):
        cc(dev["DIC"], dev["T"], dev["S"], Alk=dev["Alk"], output="pHt")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    l0 = lib.obgc_kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        e0.record(stream)
        for _ in range(args.steps):
            out = cc(dev["DIC"], dev["T"], dev["S"], Alk=dev["Alk"], output="pHt")
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = lib.obgc_kernel_launch_count() - l0
    iters = torch.zeros(n, dtype=torch.int32, device="cuda")
    cc(dev["DIC"], dev["T"], dev["S"], Alk=dev["Alk"], output="pHt", iters=iters)
    # e2e: host arrays in, pH out, through the public call
    host = {k: v.cpu().pin_memory() for k, v in dev.items()}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2 = {k: v.to("cuda", non_blocking=True) for k, v in host.items()}
    ph = cc(d2["DIC"], d2["T"], d2["S"], Alk=d2["Alk"], output="pHt").cpu()
    e2e_s = time.perf_counter() - t0
    fpeak = fp64_peak()
    bytes_per_cell = 4 * 8 + 8
    achieved = CARBON_FLOP_PER_CELL * n / (ms / 1e3) / 1e9
    line = {
        "metric": "carbonate-system solves/s", "value": n / (ms / 1e3), "unit": "cells/s", "n_gpus": 1,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded LOBSTER DIC/Alk/T/S)",
        "config": {"workload": "pH (total scale) of every cell, DIC/Alk/T/S of the LOBSTER 3-D state, FP64 damped "
                               "Newton with the bisection guard", "cells": n,
                   "newton_iterations": {"mean": float(iters.double().mean()), "max": int(iters.max())},
                   "pH_range": [float(ph.min()), float(ph.max())]},
        "e2e": {"value": n / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": 4 * 8 * n, "d2h_bytes_per_step": 8 * n},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": fpeak, "unit": "GFLOP/s", "frac": achieved / fpeak,
                     "traffic": bytes_per_cell * n, "peak_source": "measured (obgc_fp64_fma_peak, FP64 FMA chains)",
                     "kernel": "carbon_kernel", "flop_per_cell": CARBON_FLOP_PER_CELL,
                     "note": "FLOPs per cell from ncu sass counters; the FP64 pipe also issues compares and "
                             "conversions, so pipe-busy exceeds frac"},
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- PISCES 3-D
PIS_SHAPE = (128, 128, 48)
PIS_EXTENT = (100_000.0, 100_000.0, 1000.0)
PIS_DT = 1200.0
PIS_SURFACE_PAR = 100.0
PIS_WORKLOAD = ("PISCES 3-D, 128x128x48 (100 km x 100 km x 1000 m), 26 tracers, MultiBand PAR (3 bands, surface "
                "100 W/m2), WENO5 + POC/GOC sinking + RK3, calcite saturation FP64, dt=1200 s")


def pisces_cpu_baseline(threads=None, steps=None):
    """The oracle's FP64 PISCES model (or_pisces_step3d) on a 64x64x48 sub-domain, all host threads."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import obgc
    from obgc import _abi as A
    from obgc.light import MultiBandPhotosyntheticallyActiveRadiation
    threads = threads or (os.cpu_count() or 1)
    shape = (64, 64, 48)
    g = obgc.RectilinearGrid(shape, (PIS_EXTENT[0] * shape[0] / PIS_SHAPE[0], PIS_EXTENT[1] * shape[1] / PIS_SHAPE[1],
                                     PIS_EXTENT[2]), ("Periodic", "Periodic", "Bounded"))
    bgc = obgc.PISCES(g)
    light = MultiBandPhotosyntheticallyActiveRadiation(grid=g, surface_PAR=PIS_SURFACE_PAR)
    m = O.pisces3d(bgc.params, g.c_grid(), light, -50.0, surface_kind=A.SURFACE_CONSTANT, surface_value=PIS_SURFACE_PAR)
    init = obgc.pisces_initial_conditions(g, seed=5)
    st = np.ascontiguousarray(np.stack([init[n] for n in A.PISCES_ASCII]).reshape(26, -1))
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=0, device="cpu")
    u = u.numpy().ravel().copy()
    v = v.numpy().ravel().copy()
    O.pisces_step3d(m, st, u=u, v=v, t=0.0, dt=PIS_DT, nsteps=1, threads=threads)   # warm
    if steps is None:
        t0 = time.perf_counter()
        O.pisces_step3d(m, st, u=u, v=v, t=PIS_DT, dt=PIS_DT, nsteps=1, threads=threads)
        one = time.perf_counter() - t0
        steps = max(1, min(30, int(15.0 / max(one, 1e-3))))
    t0 = time.perf_counter()
    O.pisces_step3d(m, st, u=u, v=v, t=2 * PIS_DT, dt=PIS_DT, nsteps=steps, threads=threads)
    el = time.perf_counter() - t0
    return {"value": 26 * g.N * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} RK3 steps of a 64x64x48 PISCES sub-domain (26 tracers), FP64, {el:.1f} s"}, el / steps


def run_pisces(args):
    """26-tracer PISCES 3-D model: update_biogeochemical_state! (MultiBand light, euphotic depth,
    mixed-layer PAR, calcite saturation) + the PISCES functor + the fused WENO5/sinking/RK3 substep,
    three stages per step, state resident in HBM."""
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    torch.cuda.set_device(0)
    lib = A.load()
    prec = args.precision if args.precision != "f64" else "mixed"
    shape = tuple(args.shape) if args.shape else PIS_SHAPE
    g = obgc.RectilinearGrid(shape, (PIS_EXTENT[0] * shape[0] / PIS_SHAPE[0], PIS_EXTENT[1] * shape[1] / PIS_SHAPE[1],
                                     PIS_EXTENT[2]), ("Periodic", "Periodic", "Bounded"),
                             dtype="f32" if prec == "f32" else "f64")
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=7)
    model = obgc.PiscesModel(g, biogeochemistry=obgc.PISCES(g), velocities=(u, v), precision=prec,
                             mixed_layer_depth=-50.0, surface_PAR=PIS_SURFACE_PAR)
    model.set_(**obgc.pisces_initial_conditions(g, seed=5))
    for _ in range(max(args.warmup, 3)):
        model.time_step(PIS_DT)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    model.set_profiling(True)
    l0 = lib.obgc_kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        e0.record(stream)
        model.time_step(PIS_DT, nsteps=args.steps, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = lib.obgc_kernel_launch_count() - l0
    phases = model.last_timing()
    model.set_profiling(False)
    value = 26 * g.N * args.steps / (ms / 1e3)
    finite = all(bool(torch.isfinite(model.tracers[n]).all()) for n in A.PISCES_TRACERS)

    # e2e: pinned host state in, one step, state out, through the public model call; two ensemble
    # members alternate, as for the headline workload
    member2 = obgc.PiscesModel(g, biogeochemistry=obgc.PISCES(g), velocities=(u, v), precision=prec,
                               mixed_layer_depth=-50.0, surface_PAR=PIS_SURFACE_PAR)
    member2.set_(**obgc.pisces_initial_conditions(g, seed=6))
    member2.time_step(PIS_DT)
    members = []
    for mdl in (model, member2):
        host = {n: torch.empty(g.shape, dtype=mdl.dtype, pin_memory=True) for n in A.PISCES_TRACERS}
        for n in A.PISCES_TRACERS:
            host[n].copy_(mdl.tracers[n])
        members.append(((lambda mdl=mdl: mdl.time_step(PIS_DT, stream=stream.cuda_stream)),
                        {n: mdl.tracers[n] for n in A.PISCES_TRACERS}, host))
    torch.cuda.synchronize()
    e2e_steps = max(4, min(args.steps, 10))
    h2d = sum(h.numel() * h.element_size() for h in members[0][2].values())
    e2e_ms = e2e_members_ms(members, e2e_steps, stream)
    del member2, members

    # roofline of the dominant phase (algorithmic bytes per cell of one stage, state precision s,
    # tendency precision 4): functor reads 26 tracers + PAR x4 + Omega and writes 24 tendencies;
    # substep reads 26 tracers + 24 functor tendencies + 26 previous tendencies + u, v and writes
    # 26 tracers + 26 tendencies; calcite reads DIC Alk T S Si + H (f64) and writes Omega + H
    s = 4 if prec == "f32" else 8
    per_cell = {"functor": 31 * s + 24 * 4, "substep": 54 * s + 76 * 4, "calcite": 6 * s + 16,
                "light": 0}
    stages = max(phases["stages"], 1)
    dom = max(("functor", "substep", "calcite", "light"), key=lambda k: phases[k])
    avg_ms = phases[dom] / stages
    peak, peak_kind = peaks()
    achieved = per_cell[dom] * g.N / (avg_ms / 1e3) / 1e9 if per_cell[dom] else 0.0
    if dom == "calcite":
        fpeak = fp64_peak()
        roof = {"bound": "fp64", "achieved": OMEGA_FLOP_PER_CELL * g.N / (avg_ms / 1e3) / 1e9, "peak": fpeak,
                "unit": "GFLOP/s", "peak_source": "measured (obgc_fp64_fma_peak, FP64 FMA chains)",
                "traffic": per_cell[dom] * g.N, "flop_per_cell": OMEGA_FLOP_PER_CELL}
        roof["frac"] = roof["achieved"] / fpeak
    else:
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "peak_source": peak_kind}
    cpu = None
    if not args.no_cpu_baseline:
        cpu, _ = pisces_cpu_baseline()
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if prec == "f32" else "f64-state/f32-compute",
        "data": "synthetic (seeded PISCES depth profiles with 5% correlated lognormal noise, random-streamfunction velocity)",
        "config": {"workload": PIS_WORKLOAD if shape == PIS_SHAPE else PIS_WORKLOAD.replace("128x128x48", "x".join(map(str, shape))),
                   "grid": list(shape), "tracers": 26, "dt_s": PIS_DT, "precision": prec,
                   "l2": "working set per stage (state, tendencies, functor tendencies, PAR, Omega, H: %.0f MB) larger "
                         "than L2 (129 MB)" % ((26 * s + 26 * 4 + 24 * 4 + 6 * s + 8) * g.N / 1e6), "finite": finite,
                   "phase_ms_per_step": {k: phases[k] / args.steps for k in ("light", "calcite", "functor", "substep")}},
        "e2e": {"value": 26 * g.N / (e2e_ms / 1e3), "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d, "ms_per_step": e2e_ms, "steps": e2e_steps,
                "pipeline": "2 ensemble members alternate: each step copies its member's state in from pinned "
                            "host memory and back; a member's copies overlap the other's step"},
        "gpu_launches": int(launches),
        "roofline": {**roof, "kernel": {"functor": "pisces_kernel",
                     "substep": "substep_kernel<V_EXTERNAL,26>", "calcite": "pisces_omega_kernel",
                     "light": "multiband light"}[dom], "algorithmic_bytes_per_launch": per_cell[dom] * g.N,
                     "avg_launch_ms": avg_ms},
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- NPZD 2-D front
FRONT_WORKLOAD = ("NPZD 2-D buoyancy front (README.md:41-52), 160x32 over 10 km x 500 m, Bounded/Flat/Bounded, "
                  "N P Z D + T, WENO5 with zero velocity + sinking + TwoBand PAR + RK3, dt = 50 s, 2000 steps, FP64")


def run_front(args):
    """The reference's README example as one 2000-step run: launch-latency bound (5,120 cells), so
    the steps replay from one CUDA graph."""
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    torch.cuda.set_device(0)
    lib = A.load()
    g = obgc.RectilinearGrid((160, 32), (10000.0, 500.0), ("Bounded", "Flat", "Bounded"))
    bgc = obgc.NPZD(g)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, precision="f64")
    if args.tz:
        model.set_tiling(args.tz)
    init = obgc.npzd_front_initial_conditions(g)
    dt, nsteps = 50.0, 2000
    obgc.set_(model, **init)
    s0 = {n: model.tracers[n].clone() for n in model.tracer_names}
    for _ in range(max(args.warmup, 3)):
        obgc.time_step(model, dt, nsteps=nsteps, graph=True)
    stream = torch.cuda.current_stream()
    times = []
    l0 = lib.obgc_kernel_launch_count()
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            for n in model.tracer_names:
                model.tracers[n].copy_(s0[n])
            model.clock.time = 0.0
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            obgc.time_step(model, dt, nsteps=nsteps, graph=True)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    launches = (lib.obgc_kernel_launch_count() - l0) // max(args.steps, 1)
    ms = float(np.median(times))
    nt = len(model.tracer_names)
    got = model.state_array().cpu().numpy()
    # end to end: the initial state from pinned host memory, the run, the state back
    host = {n: s0[n].cpu().pin_memory() for n in model.tracer_names}
    out = {n: torch.empty_like(host[n]).pin_memory() for n in model.tracer_names}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for n in model.tracer_names:
        model.tracers[n].copy_(host[n], non_blocking=True)
    model.clock.time = 0.0
    obgc.time_step(model, dt, nsteps=nsteps, graph=True)
    for n in model.tracer_names:
        out[n].copy_(model.tracers[n], non_blocking=True)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    # the oracle: the same run on one host thread, its error statement and its time
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names)
    ref = np.ascontiguousarray(np.stack([s0[n].cpu().numpy() for n in model.tracer_names]))
    t0 = time.perf_counter()
    O.step3d(m, ref, t=0.0, dt=dt, nsteps=nsteps, threads=1)
    cpu_s = time.perf_counter() - t0
    err = {n: float(np.max(np.abs(got[q] - ref[q])) / max(np.max(np.abs(ref[q])), 1e-300))
           for q, n in enumerate(model.tracer_names)}
    updates = nt * g.N * nsteps
    line = {
        "metric": METRIC, "value": updates / (ms / 1e3), "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / nsteps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "the reference README's initial conditions",
        "config": {"workload": FRONT_WORKLOAD, "ms_per_run": ms, "max_rel_err_vs_oracle": max(err.values()),
                   "l2": "5,120 cells: resident in L2 (launch-latency bound; each timed run restarts from the initial state)"},
        "e2e": {"value": updates / (e2e_ms / 1e3), "unit": METRIC, "h2d_bytes_per_step": nt * g.N * 8 / nsteps,
                "d2h_bytes_per_step": nt * g.N * 8 / nsteps, "ms_per_run": e2e_ms},
        "gpu_launches": int(launches),
        "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None,
                     "note": "5,120 cells occupy a fraction of one wave: the run is bound by the 6,000 dependent "
                             "substep launches replayed from a CUDA graph"},
        "clocks": clocks.summary(),
        "cpu_baseline": {"value": updates / cpu_s, "unit": METRIC, "cores": 1, "kind": "port",
                         "sample": f"the whole 2000-step run on one host thread, FP64, {cpu_s:.1f} s"},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- BoxModel
BOX_REF_MS = 23.523     # benchmark/box_model.jl:67: 1000 NPZD steps of 20 min, no output
BOX_WORKLOAD = ("NPZD BoxModel (benchmark/box_model.jl): N=10, P=0.1, Z=0.01, PAR = PAR0(t) exp(0.2 z) at z = -10 m, "
                "RK3, dt = 20 min, 1000 steps, FP64")


def _box_par(t):
    import math
    year, day = 365 * 86400.0, 86400.0
    par0 = 60 * (1 - math.cos((t + 15 * day) * 2 * math.pi / year)) * \
        (1 / (1 + 0.2 * math.exp(-(((t % year) - 200 * day) / (50 * day)) ** 2))) + 2
    return par0 * math.exp(0.2 * -10)


def run_box(args):
    """The reference's BoxModel benchmark: one NPZD box model, 1000 RK3 steps of 20 minutes, in one
    launch; plus an ensemble of 16,384 such boxes (parameter-calibration style) for throughput."""
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    torch.cuda.set_device(0)
    lib = A.load()
    g = obgc.BoxModelGrid()
    bgc = obgc.NPZD(g, light_attenuation=obgc.PrescribedPhotosyntheticallyActiveRadiation(_box_par))
    dt, nsteps = 1200.0, 1000
    init = {"N": 10.0, "P": 0.1, "Z": 0.01}

    def fresh(n):
        box = obgc.BoxModel(bgc, n_models=n, precision="f64")
        box.set(**init)
        return box

    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 3)):
        fresh(1).run(dt, nsteps)
    torch.cuda.synchronize()
    # device time of the 1000-step launch, and the run end to end through BoxModel.run (PAR sampled
    # at every stage on the host, uploaded, the run, the state read back)
    dev_ms, e2e_ms = [], []
    l0 = lib.obgc_kernel_launch_count()
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            box = fresh(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            box.run(dt, nsteps)
            e1.record(stream)
            state = box.state.cpu()
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
            dev_ms.append(e0.elapsed_time(e1))
    launches = lib.obgc_kernel_launch_count() - l0
    dev = float(np.median(dev_ms))
    e2e = float(np.median(e2e_ms))
    # parity with the oracle on the same stage PAR
    import oracle as O
    stages = np.array([_box_par(dt * (k + c)) for k in range(nsteps) for c in (0, 8 / 15, 2 / 3)])
    ref = O.box_run(bgc.params, {A.NAME_INDEX[k]: v for k, v in init.items()}, dt, nsteps, PAR_stages=stages)
    got = state.numpy()[0]
    err = float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300 + 1e-12 * np.max(np.abs(ref)))))
    # ensemble throughput
    n_ens = 16384
    ens = fresh(n_ens)
    ens.run(dt, 10)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ens.run(dt, nsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    ens_ms = e0.elapsed_time(e1)
    # CPU: the oracle, one box, 1000 steps, one thread
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 2.0:
        O.box_run(bgc.params, {A.NAME_INDEX[k]: v for k, v in init.items()}, dt, nsteps, PAR_stages=stages)
        reps += 1
    cpu_ms = (time.perf_counter() - t0) * 1e3 / reps
    line = {
        "metric": "ms per 1000-step NPZD BoxModel run", "value": dev, "unit": "ms", "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": dev / nsteps, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": dev / BOX_REF_MS, "dtype": "f64", "data": "the reference benchmark's own inputs",
        "config": {"workload": BOX_WORKLOAD, "published_ms": BOX_REF_MS, "max_rel_err_vs_oracle": err,
                   "ensemble": {"boxes": n_ens, "ms_per_1000_steps": ens_ms,
                                "box_steps_per_s": n_ens * nsteps / (ens_ms / 1e3)}},
        "e2e": {"value": e2e, "unit": "ms", "h2d_bytes_per_step": stages.nbytes / nsteps + 8 * A.NUM_NAMED / nsteps,
                "d2h_bytes_per_step": 8 * A.NUM_NAMED / nsteps},
        "gpu_launches": int(launches),
        "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None,
                     "note": "one thread integrates the box's 3000 dependent RK3 stages; no bandwidth or pipe bound "
                             "applies to a single box, the ensemble line carries the throughput"},
        "clocks": clocks.summary(),
        "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": 1, "kind": "port",
                         "sample": f"{reps} runs of the oracle's box integrator (1 box, 1000 steps), FP64"},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- OAE replicates
OAE_WORKLOAD = ("OAE experiment at the headline grid: LOBSTER + CarbonateSystem(2) (DIC1 DIC2 Alk1 Alk2) + T S, "
                "256x256x64, a CO2 gas-exchange condition on each replicate (5 m/s), an alkalinity release into "
                "Alk2 in a surface disc, WENO5 + sinking + TwoBand PAR + RK3, dt=300 s")


def run_oae(args):
    """examples/oae_experiment.jl's tracer physics at the headline grid: the replicates DIC2 / Alk2
    run as passive launches with the DIC / Alk tendency, two gas-exchange flux kernels per stage,
    the release as a windowed forcing field."""
    import numpy as np
    import torch
    import obgc
    from obgc import _abi as A
    torch.cuda.set_device(0)
    lib = A.load()
    prec = args.precision
    shape = tuple(args.shape) if args.shape else SHAPE
    g = obgc.RectilinearGrid(shape, (EXTENT[0] * shape[0] / SHAPE[0], EXTENT[1] * shape[1] / SHAPE[1], EXTENT[2]),
                             ("Periodic", "Periodic", "Bounded"), dtype="f32" if prec == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(2))
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=7)
    bcs = {f"DIC{r}": obgc.CarbonDioxideGasExchangeBoundaryCondition(
        wind_speed=5.0, water_concentration=obgc.CarbonDioxideConcentration(DIC=f"DIC{r}", Alk=f"Alk{r}")) for r in (1, 2)}
    z, y, x = g.nodes()
    disc = ((x[None, None, :] - g.Lx / 2) ** 2 + (y[None, :, None] - g.Ly / 2) ** 2 < (g.Lx / 10) ** 2) & (z[:, None, None] > -10)
    release = obgc.Forcing(np.where(disc, 1e-3, 0.0) * np.ones(g.shape), start_time=1200.0, end_time=1200.0 + 3600.0)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision=prec,
                                     boundary_conditions=bcs, forcing={"Alk2": release})
    init = obgc.lobster_initial_conditions(g, seed=11)
    vals = {k: val for k, val in init.items() if k in model.tracers}
    vals.update(DIC1=init["DIC"], DIC2=init["DIC"], Alk1=init["Alk"], Alk2=init["Alk"])
    obgc.set_(model, **vals)
    nt = len(model.tracer_names)
    obgc.time_step(model, DT, nsteps=max(args.warmup, 3), graph=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    l0 = lib.obgc_kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        torch.cuda.synchronize()
        e0.record(stream)
        obgc.time_step(model, DT, nsteps=args.steps, graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = lib.obgc_kernel_launch_count() - l0
    t = {n: model.tracers[n].double() for n in ("DIC1", "DIC2", "Alk1", "Alk2")}
    line = {
        "metric": METRIC, "value": nt * g.N * args.steps / (ms / 1e3), "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"f32": "f32", "mixed": "f64-state/f32-compute", "f64": "f64"}[prec],
        "data": "synthetic (seeded LOBSTER initial conditions, both replicates equal at the start)",
        "config": {"workload": OAE_WORKLOAD if shape == SHAPE else OAE_WORKLOAD.replace("256x256x64", "x".join(map(str, shape))),
                   "grid": list(shape), "tracers": nt, "precision": prec, "parallelism": "1 GPU"},
        "gpu_launches": int(launches),
        "released_alkalinity_excess": float((t["Alk2"] - t["Alk1"]).sum().item()),
        "dic_uptake_excess": float((t["DIC2"] - t["DIC1"]).sum().item()),
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="lobster3d", choices=["lobster3d", "columns", "service", "carbon", "accuracy",
                                                                    "pisces", "box", "front", "oae"])
    ap.add_argument("--rates", type=float, nargs="*", default=None, help="service: Poisson arrival rates (1/s)")
    ap.add_argument("--arrival-seconds", type=float, default=2.0, help="service: seconds of arrivals per rate")
    ap.add_argument("--chunk", type=int, default=32, help="service: steps per launch")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="obgc", choices=["obgc", "reference"])
    ap.add_argument("--precision", default="f32", choices=["f32", "mixed", "f64"])
    ap.add_argument("--tz", type=int, default=0)
    ap.add_argument("--staging", default="default", choices=["default", "tma", "cp.async"],
                    help="tile staging of the fused substep (default: the library's choice)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="lobster3d: keep the library's default launch shape")
    ap.add_argument("--shape", type=int, nargs=3, default=None,
                    help="grid size for profiling a smaller case of the same kernel (default 256 256 64)")
    args = ap.parse_args()
    args.steps_given = "--steps" in sys.argv
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "columns":
        return run_columns(args)
    if args.workload == "carbon":
        return run_carbon(args)
    if args.workload == "pisces":
        return run_pisces(args)
    if args.workload == "box":
        return run_box(args)
    if args.workload == "front":
        return run_front(args)
    if args.workload == "accuracy":
        return run_accuracy(args)
    if args.workload == "oae":
        return run_oae(args)
    if args.workload == "service":
        if "--precision" not in sys.argv:
            args.precision = "mixed"
        return run_service(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
