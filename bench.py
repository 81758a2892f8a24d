"""Benchmark: tracer-cell updates/s of 3-D LOBSTER with carbonates on one GB300.

Workload: 256 x 256 x 64 grid (50 km x 50 km x 500 m, Periodic/Periodic/Bounded), 11 advected tracers
(NO3 NH4 P Z sPOM bPOM DOM DIC Alk + T S), seeded initial conditions, a divergence-free velocity
from a seeded random streamfunction (0.1 m/s RMS), TwoBand PAR with the default surface PAR,
WENO5 advection + sinking + LOBSTER + RK3, dt = 300 s.  One tracer-cell update = one tracer
advanced one full RK3 step (three substeps) in one cell.

Arms:
  default           the fused CUDA path through the C ABI (state resident in HBM for `value`;
                    `e2e` copies the whole state host->device and back around every step).
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
METRIC = "tracer-cell updates/s"
WORKLOAD = "LOBSTER+carbonates 3-D, 256x256x64, 11 tracers, WENO5 + sinking + TwoBand PAR + RK3, dt=300 s"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


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


def cpu_baseline(steps=None, threads=None):
    """The oracle (CPU restatement of the reference's path) on a bounded sample of the workload:
    a 128 x 128 x 64 sub-domain with the same per-cell work, FP64, all host threads."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import obgc
    threads = threads or (os.cpu_count() or 1)
    shape = (128, 128, 64)
    g = obgc.RectilinearGrid(shape, (EXTENT[0] * shape[0] / SHAPE[0], EXTENT[1] * shape[1] / SHAPE[1], EXTENT[2]))
    p = O.preset("LOBSTER")
    p.carbonate_system = 1
    names = ["NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM", "DIC", "Alk", "T", "S"]
    m = O.model3d(p, g.c_grid(), names)
    init = obgc.lobster_initial_conditions(g, seed=1)
    st = np.ascontiguousarray(np.stack([np.broadcast_to(np.asarray(init[n], dtype=np.float64), g.shape) for n in names]))
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=0, device="cpu")
    u = u.numpy().ravel().copy()
    v = v.numpy().ravel().copy()
    O.step3d(m, st, u=u, v=v, t=0.0, dt=DT, nsteps=1, threads=threads)   # warm
    if steps is None:
        t0 = time.perf_counter()
        O.step3d(m, st, u=u, v=v, t=DT, dt=DT, nsteps=1, threads=threads)
        one = time.perf_counter() - t0
        steps = max(1, min(30, int(15.0 / max(one, 1e-3))))
    t0 = time.perf_counter()
    O.step3d(m, st, u=u, v=v, t=2 * DT, dt=DT, nsteps=steps, threads=threads)
    el = time.perf_counter() - t0
    value = N_TRACERS * g.N * steps / el
    return {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} RK3 steps of a 128x128x64 LOBSTER+carbonates sub-domain (11 tracers), FP64, "
                      f"{el:.1f} s"}, el / steps


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    base, per_step = cpu_baseline()
    # K timed steps of the bounded sample after W warm-up steps
    import numpy as np   # noqa: F401
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": base["sample"], "parallelism": "host threads"},
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
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=11 + rank))
    assert len(model.tracer_names) == N_TRACERS

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
    model.set_profiling(False)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = t.item()
    updates = N_TRACERS * g.N * args.steps * world
    value = updates / (ms / 1e3)

    # ---- e2e: public API with host buffers: pinned state -> device, one step, state -> host
    names = model.tracer_names
    host = {n: torch.empty(g.shape, dtype=model.state_dtype, pin_memory=True) for n in names}
    for n in names:
        host[n].copy_(model.tracers[n])
    barrier()
    e2e_steps = max(1, min(args.steps, 20))
    h2d = sum(h.numel() * h.element_size() for h in host.values())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        for n in names:
            model.tracers[n].copy_(host[n], non_blocking=True)
        obgc.time_step(model, DT, nsteps=1, graph=True)
        for n in names:
            host[n].copy_(model.tracers[n], non_blocking=True)
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_value = N_TRACERS * g.N * world / (e2e_ms / 1e3)

    # ---- roofline of the fused substep kernel
    s = 4 if prec == "f32" else 8
    gb = 4 if prec != "f64" else 8
    bytes_per_update = algorithmic_bytes_per_update(s, gb, s, N_TRACERS, 2)
    substep_avg_ms = substep_ms / (3 * args.steps) if substep_ms > 0 else ms / (3 * args.steps)
    bytes_per_launch = bytes_per_update * N_TRACERS * g.N / 3
    achieved = bytes_per_launch / (substep_avg_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "substep_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        traffic = tj.get(prec)

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
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "ms_per_step": e2e_ms},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "substep_kernel", "algorithmic_bytes_per_launch": bytes_per_launch,
                         "avg_launch_ms": substep_avg_ms},
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="obgc", choices=["obgc", "reference"])
    ap.add_argument("--precision", default="f32", choices=["f32", "mixed", "f64"])
    ap.add_argument("--tz", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shape", type=int, nargs=3, default=None,
                    help="grid size for profiling a smaller case of the same kernel (default 256 256 64)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
