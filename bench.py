"""Benchmark of the explicit time step on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
                    [--workload c1_3d_evp] [--impl reference]

A "step" is one explicit time step (the body of the reference's time loop,
dynearthsol.cxx:325-361) over the whole mesh.  The default workload is the
3D 100x100x10 km box of 80x80x26 cubes x 6 = 998,400 tetrahedra (177,147
nodes), Maxwell visco-elasto-plastic with Arrhenius viscosity and
Mohr-Coulomb plasticity, thermal diffusion on.  Its device state (~310 MB)
is larger than the 129 MB L2, so consecutive steps stream from HBM.

Metric: Mtet-steps/s = nelem x steps / time (higher is better).
* value:   device-resident state, the CUDA-graph step replayed K times, timed
           with CUDA events on the library's stream, max over ranks;
* e2e:     the drop-in call des_step_host with the state in pinned host
           memory in the reference's layout, uploaded and downloaded every
           step (host<->device copies inside the timed region);
* roofline: the dominant kernel (update_stress) timed alone with CUDA
           events: algorithmic bytes per launch / duration against the
           measured HBM copy bandwidth (MEASURED_PEAKS.json); beside it,
           fp64_pipe: its FP64 instructions per element (from the committed
           ncu capture) per second against 2 per SM per clock, the roof that
           binds on GB300;
* cpu_baseline: the reference's own step (its fields/geometry/rheology/bc/
           matprops objects compiled -O2 -fopenmp from its staged sources,
           oracle/_ref) on this host's cores, at all threads and at one
           thread, on a bounded sample of the same workload, with the oracle
           (C restatement) beside it;
--impl reference times the reference's OpenMP step alone on the same workload.
With --gpus N > 1 (torchrun) every rank runs an independent replica
(the path has no data-path exchange on one GPU per replica): "weak" scaling.
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

# bytes per element of update_stress that must cross HBM once per launch:
# reads stress, strain, strain_rate (3 x 48), plstrain, delta_plstrain,
# stressyy, edvoldt, volume, volume_old (6 x 8), connectivity (16);
# writes stress, strain, strain_rate (3 x 48), plstrain, delta_plstrain,
# stressyy, dpressure (4 x 8); node temperatures are counted per node.
STRESS_BYTES_PER_ELEM_FP64 = 3 * 48 + 6 * 8 + 16 + 3 * 48 + 4 * 8
# compulsory bytes of a whole step per tet (3D FP64): element state read and
# written once, support lists read once, node state read and written once
STEP_ELEM_BYTES = 16 + 96 + 96 + 16 + 16          # conn, stress r/w, strain r/w, plstrain r/w, volume old/new
SUPPORT_BYTES_PER_ELEM = 16
NODE_BYTES = 48 + 48 + 16 + 4                       # coord r/w, vel r/w, T r/w, bcflag


def step_bytes_per_tet(nn, ne):
    return STEP_ELEM_BYTES + SUPPORT_BYTES_PER_ELEM + (NODE_BYTES + 4) * nn / ne


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_value(kernel: str, workload: str, key: str):
    """A per-launch figure recorded from an ncu capture in profiles/
    ("key: value" line of the kernel's summary)."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":", 1)[1].split()[0])
    return None


def profile_traffic(kernel: str, workload: str):
    """dram bytes per launch recorded from an ncu capture in profiles/."""
    return profile_value(kernel, workload, "traffic_bytes_per_launch")


SM_COUNT = 152          # GB300
FP64_PER_SM_CLK = 2     # FP64 thread instructions per SM per clock (ncu peak_sustained of DFMA)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
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
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def port_baseline(wl, st, cp, clock, nthreads, budget_s=12.0):
    """Oracle (CPU restatement, OpenMP) on the same workload: a bounded
    number of steps sized to ~budget_s seconds."""
    from oracle.oracle import Oracle, state_copy
    s = state_copy(st)
    o = Oracle(wl, s, cp, nthreads, clock)
    t0 = time.perf_counter()
    o.run(2)
    t_cal = (time.perf_counter() - t0) / 2
    nsteps = int(max(2, min(200, budget_s / max(t_cal, 1e-6))))
    t0 = time.perf_counter()
    rc = o.run(nsteps)
    dt = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"oracle run failed ({rc})")
    return {"value": wl.mesh.nelem * nsteps / dt / 1e6, "unit": "Mtet-steps/s", "cores": nthreads,
            "kind": "port",
            "sample": f"{nsteps} steps of the full {wl.mesh.nelem:,}-tet workload, "
                      f"OpenMP x{nthreads} (two-colour element bands), {dt:.1f} s"}


def reference_sensitivity(wl, init, clock, cp, nsteps, fp64_final):
    """How far the reference's own algorithm moves, over the same steps from
    the same state, when its libm results move by +-1 ulp: the oracle (the
    CPU restatement, OpenMP) run twice, once as built and once with every
    transcendental result moved by -1, 0 or +1 ulp (liboracle_pert.so, one
    xorshift stream per thread).  With the default damping this sets the
    scale of any two faithful implementations' difference, the mixed step's
    against the FP64 step's included; the device FP64 step's distance from
    the plain oracle is reported beside it."""
    from oracle.oracle import Oracle, state_copy
    nth = os.cpu_count() or 1
    t0 = time.perf_counter()
    runs = []
    used = nth
    for seed in (None, 12345):
        s = state_copy(init)
        o = Oracle(wl, s, cp, nth, clock, perturb_seed=seed)
        used = o.threads
        if o.run(nsteps):
            raise RuntimeError("oracle run failed")
        runs.append(s["stress"])
    plain, pert = runs

    def l2(x, y):
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))
    return {"steps": nsteps, "oracle_vs_oracle_pm1ulp_stress_rel_l2": l2(pert, plain),
            "fp64_device_vs_oracle_stress_rel_l2": l2(fp64_final["stress"], plain),
            "sample": f"the oracle on {used} host threads, {time.perf_counter() - t0:.1f} s for both runs"}


def reference_cpu():
    """The reference's own step compiled with OpenMP (oracle/_ref), or None
    where its sources are not staged."""
    from oracle.oracle import Reference, reference_sources_available
    if not reference_sources_available():
        return None
    try:
        return Reference(3, flavour="omp")
    except OSError:
        return None


def reference_timed(ref, wl, st, cp, clock, nthreads, budget_s):
    """The reference's loop body (dynearthsol.cxx:325-361, its own fields,
    geometry, rheology, bc and matprops objects built -O2 -fopenmp) on
    nthreads OpenMP threads, for a number of steps sized to ~budget_s
    seconds: (Mtet-steps/s, steps, seconds of the loop alone)."""
    from oracle.oracle import state_copy
    ref.set_threads(nthreads)
    _, t_cal = ref.run_timed(wl, state_copy(st), cp, clock, 1)
    nsteps = int(max(2, min(200, budget_s / max(t_cal, 1e-6))))
    _, sec = ref.run_timed(wl, state_copy(st), cp, clock, nsteps)
    return wl.mesh.nelem * nsteps / sec / 1e6, nsteps, sec


def cpu_baseline(wl, st, cp, clock, nthreads, budget_s=12.0):
    """The reference's own OpenMP step on this host's cores (kind
    "reference"), at all threads and at 1 thread, with the oracle port beside
    it; the port alone where the reference's sources are not staged."""
    port = port_baseline(wl, st, cp, clock, nthreads, budget_s)
    ref = reference_cpu()
    if ref is None:
        return port
    v, n, sec = reference_timed(ref, wl, st, cp, clock, nthreads, budget_s)
    v1, n1, sec1 = reference_timed(ref, wl, st, cp, clock, 1, budget_s)
    ref.set_threads(nthreads)
    return {"value": v, "unit": "Mtet-steps/s", "cores": nthreads, "kind": "reference",
            "sample": f"{n} steps of the full {wl.mesh.nelem:,}-tet workload through the reference's own "
                      f"fields/geometry/rheology/bc/matprops objects (-O2 -fopenmp, {2 * nthreads} element "
                      f"bands), OpenMP x{nthreads}, {sec:.1f} s of loop",
            "one_thread": {"value": v1, "cores": 1, "sample": f"{n1} steps, {sec1:.1f} s of loop"},
            "port": port}


def setup_workload(name):
    from dynearthsol_gb300.config import initial_state, make_workload
    wl = make_workload(name)
    st, cp = initial_state(wl)
    return wl, st, cp


def run_reference(args, rank, world):
    """The reference's own CPU implementation of the step on this host, all
    threads: its fields/geometry/rheology/bc/matprops objects compiled with
    OpenMP from its staged sources (oracle/_ref); the oracle port where those
    are not staged."""
    if rank != 0:
        return 0
    wl, st, cp = setup_workload(args.workload)
    from oracle.oracle import Oracle, state_copy
    nthreads = os.cpu_count() or 1
    o = Oracle(wl, st, cp, nthreads)
    o.init_fields()
    clock = o.clock
    ref = reference_cpu()
    if ref is not None:
        ref.set_threads(nthreads)
        s = state_copy(st)
        clock, _ = ref.run_timed(wl, s, cp, clock, args.warmup)
        # each timed step is one explicit step of the full workload
        _, el = ref.run_timed(wl, s, cp, clock, args.steps)
        kind, what = "reference", (f"the reference's own objects (-O2 -fopenmp, {2 * nthreads} element bands), "
                                   "loop time only")
    else:
        for _ in range(args.warmup):
            o.run(1)
        t0 = time.perf_counter()
        rc = o.run(args.steps)
        el = time.perf_counter() - t0
        if rc:
            raise RuntimeError(f"oracle failed ({rc})")
        kind, what = "port", "the oracle port (the reference's sources are not staged here)"
    v = wl.mesh.nelem * args.steps / el / 1e6
    line = {
        "impl": "reference", "metric": metric_name(args), "value": v, "unit": "Mtet-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args, wl),
        "cpu_baseline": {"value": v, "unit": "Mtet-steps/s", "cores": nthreads, "kind": kind,
                         "sample": f"{args.steps} timed steps (after {args.warmup} warm-up) of the full "
                                   f"{wl.mesh.nelem:,}-tet workload, OpenMP x{nthreads}: {what}"},
        "e2e": {"value": v, "unit": "Mtet-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def metric_name(args):
    if args.precision == "mixed":
        return "Mtet-steps/s (mixed FP32/FP64 explicit step; FP64 step and stress error beside it)"
    return "Mtet-steps/s (FP64 explicit step)"


def config_of(args, wl):
    return {"workload": args.workload, "nelem": wl.mesh.nelem, "nnode": wl.mesh.nnode,
            "precision": args.precision, "physics": wl.description,
            "l2_policy": "inputs larger than L2 (device state > 129 MB), no flush",
            "parallelism": f"replicas x{args.gpus}"}


def max_over_ranks(value: float, dist, device: str = "cuda") -> float:
    """The largest of every rank's value (the job's time is its slowest
    rank's); the value itself without a process group."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(units_per_rank: float, seconds: float, world: int) -> float:
    """Whole-job throughput in millions of units per second: the units all
    ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds / 1e6


def timed_steps(m, stream, steps, warmup, dist, sample_clocks=False, local=0):
    """W untimed steps, then K steps between CUDA events on the library's
    stream (barrier + synchronize on both sides); returns (ms, launches,
    clocks)."""
    import torch
    m.step(warmup)
    m.sync()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local) if sample_clocks else None
    if sampler:
        sampler.start()
    l0 = m.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    m.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if sampler else None
    status = m.device_status()
    if status:
        raise RuntimeError(f"device status {status:#x} during the timed run")
    return max_over_ranks(ms, dist), m.launches() - l0, clocks


def error_gate(wl, init, clock0, cp, stream, nsteps):
    """Mixed vs FP64 relative L2 stress error after nsteps from the same
    state, with damping option 2 (not chaotic); gate 1e-6."""
    from dataclasses import replace
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.solver import DeviceModel
    wl2 = replace(wl, params=replace(wl.params, damping_option=2))
    out = {}
    for name, prec in (("fp64", capi.PREC_FP64), ("mixed", capi.PREC_MIXED)):
        m = DeviceModel(wl2, comp_pressure=cp, precision=prec, stream=stream.cuda_stream)
        m.upload({k: v.copy() for k, v in init.items()}, clock0)
        m.step(nsteps)
        out[name] = m.download()
        if m.device_status():
            raise RuntimeError("device status during the error gate")
        m.close()
    a, b = out["fp64"], out["mixed"]
    l2 = float(np.linalg.norm(b["stress"] - a["stress"]) / np.linalg.norm(a["stress"]))
    maxn = {k: float(np.abs(b[k] - a[k]).max() / max(np.abs(a[k]).max(), 1e-300))
            for k in ("vel", "stress", "strain", "temperature", "plstrain", "coord", "force", "volume")}
    return {"config": "same mesh and physics, damping_option 2", "steps": nsteps,
            "stress_rel_l2_err": l2, "gate": 1e-6, "passed": l2 <= 1e-6,
            "max_normalised_err": maxn,
            "yielded_elements_fp64": int((a["plstrain"] > init["plstrain"]).sum())}


def kernel_time(m, stream, fn, reps=20):
    """Average duration (ms) of one per-function entry point, CUDA events."""
    import torch
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m.call(fn)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        m.call(fn)
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="c1_3d_evp")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--gate-steps", type=int, default=2000,
                    help="steps of the damping-2 mixed-vs-FP64 stress-error gate (0: skip)")
    ap.add_argument("--adjoint-steps", type=int, default=500,
                    help="window of the adjoint benchmark (0: skip it)")
    ap.add_argument("--adjoint-every", type=int, default=50,
                    help="checkpoint spacing of the adjoint window (0: the whole window as one segment, taped by "
                         "its forward, or every 50 steps when that tape does not fit in device memory)")
    ap.add_argument("--adjoint-fd", type=int, default=20,
                    help="elements checked against central differences in the adjoint benchmark")
    ap.add_argument("--yield-spinup", type=int, default=8000,
                    help="mixed steps that bring the weak band of the yielding benchmark to yield (0: skip it)")
    ap.add_argument("--yield-adjoint-steps", type=int, default=100,
                    help="window of the adjoint with yielding elements (cohesion and friction gradients; 0: skip)")
    ap.add_argument("--heat-adjoint-steps", type=int, default=200,
                    help="window of the heat adjoint on the 4,056,000-tet jittered mesh (0: skip)")
    ap.add_argument("--scale-steps", type=int, default=1000,
                    help="steps of the 7,987,200-tet mixed-vs-FP64 run (0: skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.solver import DeviceModel

    wl, st0, cp = setup_workload(args.workload)
    ne, nn = wl.mesh.nelem, wl.mesh.nnode
    stream = torch.cuda.Stream()
    f64 = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_FP64, stream=stream.cuda_stream)
    init = f64.init_fields(st0)
    clock0 = f64.clock()
    if args.precision == "mixed":
        m = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_MIXED, stream=stream.cuda_stream)
        m.upload({k: v.copy() for k, v in init.items()}, clock0)
    else:
        m = f64

    # ---- headline: device-resident throughput of the selected precision ----
    ms, launches, clocks = timed_steps(m, stream, args.steps, args.warmup, dist, True, local)
    value = aggregate_value(ne * args.steps, ms / 1e3, world)
    compare = None
    fp64_final = None
    if args.precision == "mixed" and not args.no_compare:
        ms64, _, _ = timed_steps(f64, stream, args.steps, args.warmup, dist)
        a, b = f64.download(), m.download()
        l2 = float(np.linalg.norm(b["stress"] - a["stress"]) / np.linalg.norm(a["stress"]))
        maxn = {k: float(np.abs(b[k] - a[k]).max() / max(np.abs(a[k]).max(), 1e-300))
                for k in ("vel", "stress", "strain", "temperature", "plstrain", "coord", "force")}
        compare = {"fp64_value": aggregate_value(ne * args.steps, ms64 / 1e3, world), "fp64_ms_per_step": ms64 / args.steps,
                   "speedup_mixed_over_fp64": ms64 / ms,
                   "stress_rel_l2_err_vs_fp64": l2,
                   "gated": False,
                   "why_not_gated": ("default damping (option 1): its copysign makes the FP64 step itself "
                                     "diverge under one-ulp changes over ~100 steps; the gate is "
                                     "mixed_error_gate, damping option 2"),
                   "steps_compared": args.warmup + args.steps,
                   "max_normalised_err_vs_fp64": maxn}
        fp64_final = a

    # ---- the mixed step's stress-error gate, on the same mesh with the
    # continuous damping option 2 (with the default option 1 the reference's
    # own FP64 step is chaotic: a one-ulp libm change moves its stress by
    # ~1e-4 within ~1000 steps, so no two implementations agree there) ----
    gate = None
    if args.precision == "mixed" and not args.no_compare and args.gate_steps > 0:
        gate = error_gate(wl, init, clock0, cp, stream, args.gate_steps)

    # ---- dominant kernel alone, for the roofline: its per-function form (a
    # kernel inside the step's graph cannot be timed with events) on the state
    # the timed steps left, so that it sees the same mix of elements ----
    k_ms = kernel_time(m, stream, "update_stress")
    hbm_peak, peak_kind = measured_peaks()
    alg = STRESS_BYTES_PER_ELEM_FP64 * ne + 16 * nn
    achieved = alg / (k_ms / 1e3) / 1e9
    traffic = profile_traffic(f"update_stress_{args.precision}", args.workload)
    roofline = {"bound": "hbm", "kernel": "k_update_stress" + ("_mixed3" if args.precision == "mixed" else "<3>"),
                "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": traffic, "kernel_ms": k_ms, "algorithmic_bytes_per_launch": alg,
                "peak_kind": peak_kind}
    # the roof that binds: FP64-pipe instructions per element over the
    # kernel's live time, against 2 per SM per clock at the clock sampled
    # during the timed steps.  The committed ncu capture gives both the FP64
    # add/mul/fma count and every FP64-pipe instruction (those plus compares
    # and min/max, from the pipe's activity); the second is what occupies
    # the pipe, the first what the arithmetic needs.
    prof = f"update_stress_{args.precision}"
    fp64_pipe = profile_value(prof, args.workload, "fp64_pipe_inst_per_elem")
    fp64_arith = profile_value(prof, args.workload, "fp64_inst_per_elem")
    if fp64_pipe or fp64_arith:
        per_elem = fp64_pipe or fp64_arith
        mhz = clocks["sm_mhz"] if clocks else 2070.0
        ach = per_elem * ne / (k_ms / 1e3) / 1e9
        peak = SM_COUNT * FP64_PER_SM_CLK * mhz / 1e3
        roofline["fp64_pipe"] = {"instructions_per_elem": per_elem, "arithmetic_per_elem": fp64_arith,
                                 "achieved_ginst_s": ach, "peak_ginst_s": peak, "frac": ach / peak,
                                 "clock_mhz": mhz, "clock": "sampled" if clocks else "nominal maximum"}
    step_alg = step_bytes_per_tet(nn, ne)
    step_gbs = step_alg * ne * args.steps / (ms / 1e3) / 1e9

    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(args, m, wl, init, clock0, world, dist)
    adjoint = None
    if args.adjoint_steps > 0 and rank == 0:
        adjoint = adjoint_bench(args, stream)
    yielding = None
    if args.yield_spinup > 0 and rank == 0:
        yielding = yield_bench(args, stream)
    yield_adjoint = None
    if args.yield_adjoint_steps > 0 and rank == 0:
        yield_adjoint = yield_adjoint_bench(args, stream)
    heat_adjoint = None
    if args.heat_adjoint_steps > 0 and rank == 0:
        heat_adjoint = heat_adjoint_bench(args, stream)
    scale = None
    if args.scale_steps > 0 and rank == 0:
        scale = scale_bench(args, stream)
    if rank == 0:
        line = {
            "metric": metric_name(args), "value": value, "unit": "Mtet-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (structured box mesh, seeded; no dataset)",
            "config": config_of(args, wl),
            "roofline": roofline,
            "step_hbm": {"algorithmic_bytes_per_tet": step_alg, "achieved_gbs": step_gbs,
                         "frac": step_gbs / hbm_peak},
            "mixed_vs_fp64": compare,
            "mixed_error_gate": gate,
            "e2e": e2e,
            "yield": yielding,
            "adjoint": adjoint,
            "yield_adjoint": yield_adjoint,
            "heat_adjoint": heat_adjoint,
            "scale": scale,
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(wl, init, cp, clock0, os.cpu_count() or 1)
            if fp64_final is not None:   # beside the mixed-vs-FP64 figure it qualifies
                line["cpu_baseline"]["reference_sensitivity"] = reference_sensitivity(
                    wl, init, clock0, cp, args.warmup + args.steps, fp64_final)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    m.close()
    f64.close()
    return 0


def run_fitting_tape(win, params, spacings):
    """win.run(params) with the first checkpoint spacing in `spacings` whose
    tape (spacing + 1 step records) fits in device memory; leaves win.C at
    that spacing."""
    from dynearthsol_gb300 import capi
    for i, C in enumerate(spacings):
        win.C = C
        try:
            return win.run(params)
        except capi.DesError as ex:
            if ex.code != capi.DES_ENOMEM or i == len(spacings) - 1:
                raise


def adjoint_bench(args, stream):
    """Adjoint/forward wall-time ratio on the 998,400-tet adjoint case: a
    window of K FP64 steps (dt held) with a checkpoint every C steps (by
    default the whole window as one segment, whose tape the forward records,
    ~160 GB for 500 steps; checkpoints every 50 steps when device memory is
    short); loss =
    the top-surface velocity misfit against a target run whose log10
    viscosity field is a seeded Gaussian random field (mean 21, sd 0.5,
    correlation length 15 km), evaluated at another draw of the field.  The
    log10-viscosity gradient is checked by fourth-order central differences
    (steps of 0.05) at `adjoint_fd` elements drawn among those whose
    gradient is at least a quarter of the largest.  The differences of the
    quasi-static velocity misfit carry an absolute rounding floor (~2e-26
    per unit step over 500 steps, from the velocity differences), which a
    single element's share of the gradient exceeds by 1e4 only near the top
    of the gradient's range; the fourth-order truncation at that step is
    ~(0.05 ln 10)^4 / 30 = 6e-6 of the derivative.
    The directional derivative along the normalised gradient (unit step in
    log10 viscosity, ~1e-3 per element) carries the whole gradient's signal."""
    import torch
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.adjoint import Window, adjoint_workload, surface_velocity_misfit, top_nodes
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    from dynearthsol_gb300.adjoint import fd5_misfit
    K = args.adjoint_steps
    C = args.adjoint_every if args.adjoint_every > 0 else K
    wl, lv_t, lv_s = adjoint_workload()
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_FP64, stream=stream.cuda_stream)
    init = m.init_fields(st)
    clock0 = m.clock()
    win = Window(m, init, clock0, K, C)
    nodes = top_nodes(wl.mesh)
    LV = capi.EF_LOG10_VISC
    # the whole window as one segment when its tape fits, else every 50 steps
    target = run_fitting_tape(win, {LV: lv_t}, [C] if C < K else [K, 50])["vel"]
    C = win.C

    # timed forward (recording checkpoints) and reverse sweep
    win.set_params({LV: lv_s})
    m.upload(win.start, clock0)
    m.sync()
    t0 = time.perf_counter()
    m.adjoint_forward(K, C)
    m.sync()
    t_fwd = time.perf_counter() - t0
    fin = m.download()
    loss, seed = surface_velocity_misfit(fin["vel"], target, nodes)
    yielded = int((fin["plstrain"] > init["plstrain"] + 1e-12).sum())
    m.sync()
    t0 = time.perf_counter()
    _, grad = m.adjoint_backward({"vel": seed}, want_start=False)
    m.sync()
    t_bwd = time.perf_counter() - t0
    # the plain (graph-replayed) step over the same window, for reference
    m.upload(win.start, clock0)
    m.sync()
    t0 = time.perf_counter()
    m.step(K)
    m.sync()
    t_step = time.perf_counter() - t0
    g = grad[LV]
    rng = np.random.default_rng(2024)
    cand = np.nonzero(np.abs(g) >= 0.25 * np.abs(g).max())[0]
    fd = []
    # each difference L(+) - L(-) is formed from the two runs' velocities
    # (misfit_difference), not as the difference of two nearly equal misfits
    for e in rng.choice(cand, size=min(args.adjoint_fd, len(cand)), replace=False):
        def vel_at(t, e=e):
            lv = lv_s.copy()
            lv[e] += t
            return win.run_vel({LV: lv})
        d = fd5_misfit(vel_at, 5e-2, target, nodes)
        fd.append({"elem": int(e), "adjoint": float(g[e]), "central_fd": float(d),
                   "rel_err": float(abs(d - g[e]) / max(abs(d), abs(g[e]), 1e-300))})
    # directional derivative along the normalised gradient: the whole
    # gradient's signal, well above the rounding of the misfit
    gn = np.linalg.norm(g)
    ghat = g / gn
    dfd = fd5_misfit(lambda t: win.run_vel({LV: lv_s + t * ghat}), 1.0, target, nodes)
    gdir = {"step": 1.0, "adjoint": float(gn), "central_fd": float(dfd),
            "rel_err": float(abs(dfd - gn) / max(abs(dfd), gn))}
    # the extension velocities of the two x boundaries
    vbc0 = win.base_vbc.copy()
    vbc_fd = []
    for i in (0, 1):
        h = 1e-2 * abs(vbc0[i])
        def vel_vbc(t, i=i):
            v = vbc0.copy()
            v[i] += t
            return win.run_vel({LV: lv_s, "vbc_values": v})
        d = fd5_misfit(vel_vbc, h, target, nodes)
        a = float(grad["vbc_values"][i])
        vbc_fd.append({"boundary": ["x0", "x1"][i], "adjoint": a, "central_fd": float(d),
                       "rel_err": float(abs(d - a) / max(abs(d), abs(a), 1e-300))})
    win.set_params({"vbc_values": vbc0})
    m.close()
    return {"workload": "c3_3d_adjoint", "nelem": wl.mesh.nelem, "window_steps": K, "checkpoint_every": C,
            "mode": ("one segment, taped by the forward (no recompute)" if C >= K
                     else "checkpointed; each segment recomputed onto the tape"),
            "loss": loss, "yielded_elements": yielded, "forward_s": t_fwd, "adjoint_s": t_bwd, "adjoint_over_forward": t_bwd / t_fwd,
            "graph_step_s": t_step, "adjoint_over_graph_step": t_bwd / t_step,
            "forward_and_adjoint_over_graph_step": (t_fwd + t_bwd) / t_step,
            "gradients": "log10 viscosity, shear modulus, cohesion0/1, friction0/1 per element; vbc_values",
            "vbc_grad_x": [float(grad["vbc_values"][0]), float(grad["vbc_values"][1])],
            "vbc_fd_check": vbc_fd,
            "fd_check": fd, "fd_max_rel_err": max((r["rel_err"] for r in fd), default=None),
            "fd": "fourth-order central differences, each L(+) - L(-) formed from the velocities",
            "fd_gradient_direction": gdir,
            "dt": "held at the start value (compute_dt not called in the window)",
            "damping_option": 2}


def yield_adjoint_bench(args, stream):
    """The adjoint through yielding elements: the 3D workload's physics on
    20x20x6 cubes (14,400 tets) with a band of weak material (per-element
    cohesion and friction), damping option 2, run 1000 steps until the band
    yields; then a window of K steps (checkpoint every K/5) whose loss is
    the top-surface velocity misfit against a run with the band's cohesion1
    perturbed by +-20 %.  Checks:
    * the window's gradients against the chain of K one-step adjoints
      (Window.chained_gradients: each step re-run alone from the state the
      forward reached and reversed with its end state's adjoint as the seed),
      which is the K-step adjoint by the chain rule;
    * the chain's last link (one step from the state at step K-1, the misfit
      as the loss) by fourth-order central differences: 5 entries each of
      cohesion0/1 and friction0/1 at elements yielding in that step whose
      gradient is at least 1% of the largest (an entry off by more than
      1e-6 is taken again at a tenth of the step: a kink of the return map
      inside the stencil), and along the normalised cohesion1 gradient.
    Over the whole window central differences are not a check: with
    elements on the yield surface the forward's rounding (stresses near
    1e8 Pa returned to the surface, increments near 0.1 Pa) makes the loss
    rough at every usable step size."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.adjoint import (Window, fd5_misfit, surface_velocity_misfit, top_nodes,
                                           yielding_adjoint_workload)
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    K = args.yield_adjoint_steps
    C = max(1, K // 5)
    wl, c1_t, c1_s = yielding_adjoint_workload()
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_FP64, stream=stream.cuda_stream)
    m.init_fields(st)
    m.step(1000)
    start = m.download()
    clock = m.clock()
    win = Window(m, start, clock, K, C)
    nodes = top_nodes(wl.mesh)
    C1, C0, F0, F1 = capi.EF_COHESION1, capi.EF_COHESION0, capi.EF_FRICTION0, capi.EF_FRICTION1
    names = ((C0, "cohesion0"), (C1, "cohesion1"), (F0, "friction0"), (F1, "friction1"))
    target = win.run({C1: c1_t})["vel"]
    win.set_params({C1: c1_s})
    m.upload(win.start, clock)
    m.sync()
    t0 = time.perf_counter()
    m.adjoint_forward(K, C)
    m.sync()
    t_fwd = time.perf_counter() - t0
    fin = m.download()
    yielding = np.nonzero(fin["plstrain"] > start["plstrain"] + 1e-12)[0]
    loss, seed = surface_velocity_misfit(fin["vel"], target, nodes)
    t0 = time.perf_counter()
    _, grad = m.adjoint_backward({"vel": seed}, want_start=False)
    m.sync()
    t_bwd = time.perf_counter() - t0
    # the chain of K one-step adjoints
    t0 = time.perf_counter()
    fin_c, _, g_c = win.chained_gradients({"vel": seed})
    t_chain = time.perf_counter() - t0
    chain = {n: float(np.abs(g_c[k] - grad[k]).max() / max(np.abs(grad[k]).max(), 1e-300)) for k, n in names}
    same_final = all(np.array_equal(fin_c[k], fin[k]) for k in ("vel", "stress", "plstrain", "coord"))
    # the last link: one step from the state at step K-1
    pre = Window(m, start, clock, K - 1, K - 1).run() if K > 1 else start
    link = Window(m, pre, m.clock() if K > 1 else clock, 1, 1)
    base = {k: win.fields[k].copy() for k in (C0, C1, F0, F1)}
    link.set_params(base)
    fin1 = link.run()
    y1 = np.nonzero(fin1["plstrain"] > pre["plstrain"] + 1e-12)[0]
    _, seed1 = surface_velocity_misfit(fin1["vel"], target, nodes)
    _, g1 = link.gradients({"vel": seed1})
    rng = np.random.default_rng(7)
    checks = []
    for key, name, h in ((C1, "cohesion1", 1e3), (C0, "cohesion0", 1e3), (F1, "friction1", 1e-2),
                         (F0, "friction0", 1e-2)):
        g = g1[key]
        cand = y1[np.abs(g[y1]) >= 0.01 * np.abs(g[y1]).max()] if len(y1) else []
        for e in (rng.choice(cand, size=min(5, len(cand)), replace=False) if len(cand) else []):
            def vel_at(t, e=e, key=key):
                p = dict(base)
                p[key] = base[key].copy()
                p[key][e] += t
                return link.run_vel(p)
            d = fd5_misfit(vel_at, h, target, nodes)
            r = {"param": name, "elem": int(e), "adjoint": float(g[e]), "step": h, "central_fd": float(d),
                 "rel_err": float(abs(d - g[e]) / max(abs(d), abs(g[e]), 1e-300))}
            if r["rel_err"] > 1e-6:
                # a kink of the return map (yield, shear/tension, the EVP choice)
                # inside the +-2h stencil: the difference at h / 10
                d10 = fd5_misfit(vel_at, h / 10, target, nodes)
                r["central_fd_h_over_10"] = float(d10)
                r["rel_err_h_over_10"] = float(abs(d10 - g[e]) / max(abs(d10), abs(g[e]), 1e-300))
            checks.append(r)
    gl = g1[C1]
    gn = float(np.linalg.norm(gl))
    ghat = gl / gn
    dfd = fd5_misfit(lambda t: link.run_vel({**base, C1: base[C1] + t * 1e3 * ghat}), 1.0, target, nodes) / 1e3
    m.close()
    return {"workload": "3d yielding band (20x20x6 cubes x 6 = 14,400 tets, per-element cohesion/friction)",
            "start_step": 1000, "window_steps": K, "checkpoint_every": C,
            "yielded_elements_in_window": int(len(yielding)), "loss": loss,
            "forward_s": t_fwd, "adjoint_s": t_bwd, "adjoint_over_forward": t_bwd / t_fwd,
            "nonzero_gradients": {n: int((np.abs(grad[k]) > 0).sum()) for k, n in names},
            "chain_of_one_step_adjoints": {"max_rel_diff": chain, "same_final_state": same_final,
                                           "seconds": t_chain},
            "last_step_yielding_elements": int(len(y1)),
            "fd_check_last_step": checks, "fd_max_rel_err": max((r["rel_err"] for r in checks), default=None),
            "fd_max_rel_err_refined": max((r.get("rel_err_h_over_10", r["rel_err"]) for r in checks), default=None),
            "fd_cohesion1_direction_last_step": {"adjoint": gn, "central_fd": float(dfd),
                                                 "rel_err": float(abs(dfd - gn) / max(abs(dfd), gn))}}


def yield_bench(args, stream):
    """Both steps where the Mohr-Coulomb return map is active: the 3D
    workload's mesh (998,400 tets) with a 30 km band of weak material
    (cohesion 1 -> 0.1 MPa, friction 10 -> 5 degrees), spun up with the
    mixed step until the band yields, then args.steps timed steps of each
    precision from that state.  Reports the throughputs, the elements that
    yield in the window and in its last step, and the mixed step's stress
    error against the FP64 run from the same state (reported, not gated:
    the yielding reference is itself chaotic under one-ulp changes)."""
    import torch
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import initial_state, make_workload, weak_band
    from dynearthsol_gb300.solver import DeviceModel
    wl = weak_band(make_workload("c1_3d_evp"))
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_MIXED, stream=stream.cuda_stream)
    init = m.init_fields(st)
    m.step(args.yield_spinup)
    start = m.download()
    clock = m.clock()
    ne = wl.mesh.nelem
    out = {"workload": "c1_3d_evp mesh with a weak band (2 materials)", "nelem": ne,
           "spinup_steps": args.yield_spinup, "window_steps": args.steps}
    res = {}
    for name, prec in (("fp64", capi.PREC_FP64), ("mixed", capi.PREC_MIXED)):
        d = m if prec == capi.PREC_MIXED else DeviceModel(wl, comp_pressure=cp, precision=prec,
                                                          stream=stream.cuda_stream)
        d.upload({k: v.copy() for k, v in start.items()}, clock)
        d.step(args.warmup)
        d.upload({k: v.copy() for k, v in start.items()}, clock)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        d.step(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        fin = d.download()
        res[name] = fin
        out[name] = {"value": ne * args.steps / (ms / 1e3) / 1e6, "unit": "Mtet-steps/s",
                     "ms_per_step": ms / args.steps,
                     "yielded_in_window": int((fin["plstrain"] > start["plstrain"] + 1e-12).sum()),
                     "yielding_last_step": int((fin["delta_plstrain"] > 0).sum())}
        if d is not m:
            d.close()
    a, b = res["fp64"], res["mixed"]
    out["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["mixed_vs_fp64_stress_rel_l2"] = float(np.linalg.norm(b["stress"] - a["stress"]) / np.linalg.norm(a["stress"]))
    out["yielded_at_start"] = int((start["plstrain"] > init["plstrain"] + 1e-12).sum())
    m.close()
    return out


def scale_bench(args, stream):
    """The mixed step at scale: 7,987,200 tets (160x160x52 cubes x6), the 3D
    EVP physics with per-element cohesion0/1 x (1 + 0.05 N(0,1)), seeded;
    `scale_steps` steps of the mixed and of the FP64 step from the same
    state, each timed with CUDA events on the library's stream, and the
    error of every field of the mixed run against the FP64 run."""
    import torch
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import initial_state, make_workload
    from dynearthsol_gb300.solver import DeviceModel
    n = args.scale_steps
    t0 = time.perf_counter()
    wl = make_workload("c2_3d_evp_noise")
    st, cp = initial_state(wl)
    ne = wl.mesh.nelem
    f = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_FP64, stream=stream.cuda_stream)
    init = f.init_fields(st)
    clk = f.clock()
    mx = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_MIXED, stream=stream.cuda_stream)
    mx.upload(init, clk)
    t_setup = time.perf_counter() - t0
    out = {}
    for name, m in (("mixed", mx), ("fp64", f)):
        m.step(2)
        m.upload(init, clk)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        m.step(n)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"ms_per_step": ms / n, "value": ne * n / (ms / 1e3) / 1e6}
    a, b = f.download(), mx.download()
    fields = ("vel", "stress", "strain", "temperature", "plstrain", "coord", "force", "volume")
    errs = {}
    for k in fields:
        den = float(np.abs(a[k]).max()) or 1.0
        errs[k] = float(np.abs(b[k] - a[k]).max()) / den
    l2 = float(np.linalg.norm(b["stress"] - a["stress"]) / np.linalg.norm(a["stress"]))
    yielded = int((a["plstrain"] > init["plstrain"] + 1e-12).sum())
    f.close()
    mx.close()
    return {"workload": "c2_3d_evp_noise", "nelem": ne, "steps": n, "mixed": out["mixed"], "fp64": out["fp64"],
            "speedup_mixed_over_fp64": out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"],
            "stress_rel_l2_err_vs_fp64": l2, "max_normalised_err_vs_fp64": errs,
            "yielded_elements_fp64": yielded, "damping_option": wl.params.damping_option,
            "host_setup_s": t_setup}


def heat_adjoint_bench(args, stream):
    """The irregular-mesh heat case: 4,056,000 tets (130x130x40 cubes x6,
    interior nodes jittered by +-20% of the spacing, elements randomly
    permuted), EVP mechanics coupled with explicit heat (k = 3.3 W/m/K,
    cp = 1000 J/kg/K, radiogenic 1e-6 W/m^3).  1000 steps of the mixed step,
    then an FP64 window of `heat_adjoint_steps` steps (checkpoint spacing:
    the largest of K, K/2 and 50 whose tape fits in device memory)
    whose loss is the final-temperature misfit against a target run with
    conductivity 3.3 (1 + 0.2 f), f a seeded Gaussian random field
    (correlation length 15 km); gradient with respect to the per-element
    conductivity, checked along its own direction by fourth-order central
    differences."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.adjoint import Window, fd5, grf_log10_visc
    from dynearthsol_gb300.config import initial_state, make_workload
    from dynearthsol_gb300.solver import DeviceModel
    K = args.heat_adjoint_steps
    KC = capi.EF_THERM_COND
    t0 = time.perf_counter()
    wl = make_workload("c4_3d_heat_jitter")
    ne = wl.mesh.nelem
    k0 = float(wl.mat.therm_cond[0])
    wl.elem_fields = {KC: np.full(ne, k0)}
    k_target = k0 * (1 + 0.2 * (grf_log10_visc(wl.mesh, mean=0.0, sd=1.0, seed=7)))
    st, cp = initial_state(wl)
    t_setup = time.perf_counter() - t0
    m = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_FP64, stream=stream.cuda_stream)
    init = m.init_fields(st)
    mx = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_MIXED, stream=stream.cuda_stream)
    mx.upload(init, m.clock())
    mx.sync()
    t0 = time.perf_counter()
    mx.step(1000)
    mx.sync()
    t_mixed = time.perf_counter() - t0
    mid = mx.download()
    clock = mx.clock()
    mx.close()
    win = Window(m, mid, clock, K, K)
    T_target = run_fitting_tape(win, {KC: k_target}, [K, max(K // 2, 1), 50])["temperature"]
    C = win.C

    def loss_of(k):
        T = win.run({KC: k})["temperature"]
        return 0.5 * float(np.sum((T - T_target) ** 2))

    win.set_params({KC: np.full(ne, k0)})
    m.upload(win.start, clock)
    m.sync()
    t0 = time.perf_counter()
    m.adjoint_forward(K, C)
    m.sync()
    t_fwd = time.perf_counter() - t0
    T = m.download()["temperature"]
    loss = 0.5 * float(np.sum((T - T_target) ** 2))
    m.sync()
    t0 = time.perf_counter()
    _, grad = m.adjoint_backward({"temperature": T - T_target}, want_start=False)
    m.sync()
    t_bwd = time.perf_counter() - t0
    g = grad[KC]
    gn = float(np.linalg.norm(g))
    ghat = g / gn
    step = 0.01 * k0 * np.sqrt(ne)
    dfd = fd5(lambda t: loss_of(k0 + t * ghat), step)
    m.close()
    return {"workload": "c4_3d_heat_jitter", "nelem": ne, "mixed_steps_before": 1000,
            "mixed_step_s": t_mixed, "window_steps": K, "checkpoint_every": C, "loss": loss,
            "forward_s": t_fwd, "adjoint_s": t_bwd, "adjoint_over_forward": t_bwd / t_fwd,
            "gradient": "per-element thermal conductivity",
            "fd_gradient_direction": {"step_per_element_rms": 0.01 * k0, "adjoint": gn, "central_fd": dfd,
                                      "rel_err": abs(dfd - gn) / max(abs(dfd), gn)},
            "host_setup_s": t_setup}


def run_e2e(args, m, wl, init, clock0, world, dist):
    import torch
    ne = wl.mesh.nelem
    pinned = {}
    for k, v in init.items():
        tt = torch.empty(v.shape, dtype=torch.float64, pin_memory=True)
        a = tt.numpy()
        a[...] = v
        pinned[k] = (tt, a)
    hs = {k: a for k, (tt, a) in pinned.items()}
    # bytes des_step_host moves per call: every array of the state, less the
    # fields the step overwrites before reading them and, on the slab-pipelined
    # path (one step per call), the geometric fields it forms from the uploaded
    # coordinates (not uploaded), and those no step writes (not downloaded)
    total = {k: a.nbytes for k, a in hs.items() if k != "shpdy" or wl.mesh.ndims == 3}
    formed = ("volume", "shpdx", "shpdy", "shpdz", "volume_n") + (("mass",) if wl.params.is_quasi_static else ())
    h2d = sum(v for k, v in total.items()
              if k not in ("strain_rate", "force", "dpressure", "edvoldt", "ntmp") + formed)
    unwritten = ("coord0",) if wl.mat.is_plane_strain else ("coord0", "stressyy")
    d2h = sum(v for k, v in total.items() if k not in unwritten)
    clk = clock0
    for _ in range(2):
        clk = m.step_host(hs, 1, clk)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    hs = {k: a for k, (tt, a) in pinned.items()}
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        clk = m.step_host(hs, 1, clk)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = aggregate_value(ne * args.e2e_steps, max_over_ranks(e2e_s, dist), world)
    return {"value": e2e_value, "unit": "Mtet-steps/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps,
            "call": "des_step_host (pinned host state, reference AoS layout, 1 step per call)"}


if __name__ == "__main__":
    sys.exit(main())
