#!/usr/bin/env python
"""Throughput of the GB300 marker-in-cell step (markers per second).

A step is one pass of the per-timestep MIC pipeline over all markers:
  marker2nodes (per-marker physics and the per-marker visco-elasto-plastic
  + rate-and-state Newton to a 1e-10 relative residual, cell-sorted scatter,
  node tail, boundary corrections) -> interpolate_center2basic_old ->
  compute_before_solve / compute_after_solve (node RSF update) ->
  nodes2markers + moveandrotatemarkers (gather, back-scatter, RK4 advection,
  stress rotation) -> counting sort of the moved markers.
The Stokes (Pardiso) and temperature solves are outside the path; their
outputs are the seeded synthetic node fields already on the device.

Workload: the 4001 x 1001 grid with 20 markers per cell (80 M markers,
synth.make_case("c4")).  Inputs are larger than L2 (the marker arrays alone
are ~5.6 GB), so no flush is needed between steps.  Each step takes the
next time step of a seeded log-uniform sequence in [1e-3, 1e10] s.

The same steps are timed for four forms of the per-marker Newton: the
network's start with split precision (the headline `value`), the plain
start (previous slip rate) with split precision, and both starts with FP64
throughout.  Every form starts from the same uploaded state.  The start
network is first trained on the GPU on the model's own Newton problems
(collected at 8 time steps) with plain FP64 solutions as targets.

`value` is device-timed with CUDA events on the context's stream, inputs
resident in HBM.  `e2e` is the same step through the C ABI with the node
fields crossing the host boundary every step, as in the reference time loop
around its host Stokes solve: the Stokes and temperature inputs are read
back after marker2nodes asynchronously (v2c_download_node_fields_async,
copied while the node kernels run) and the solver outputs are uploaded from
pinned host memory before nodes2markers.  `newton_c3` times the Newton alone on 4 M seeded states.
`--impl reference` times the reference's own C routines (compiled from its
sources, oracle/_ref) on all host cores on a bounded window of the same
workload; the reference has no per-marker Newton.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "markers/s per MIC step, learned-guess vs plain Newton, same GPU & residual"
UNIT = "markers/s"

# algorithmic bytes per marker (FP32/int32 canonical form, each persistent
# field counted once per read and once per write; node fields spread over
# the markers per node) of the three marker sweeps:
#   m2n:  marker reads 57 B (cell, u, v, type, T, stresses, strain rates, P,
#         e, phi, velocities, cohesion, the physics results) + phi write 4 B;
#         18 node fields read, 39 written
#   n2m:  reads cell, u, v, type, T 17 B; writes the 9 updated fields 36 B;
#         19 node fields read, 15 back-scatter sums written
#   move: reads cell, u, v, type, T, sxx, sxy 25 B; writes cell, u, v, sxx,
#         sxy 20 B; 3 node fields read (vx, vy, esp; the per-quarter
#         velocity forms built from them are an intermediate, not counted)
ALG_BYTES = {"m2n": 57 + 4, "n2m": 17 + 36, "move": 25 + 20}
NODE_FIELDS = {"m2n": 18 + 39, "n2m": 19 + 15, "move": 3}
STEP_MARKER_BYTES = 57 + 48
STEP_NODE_FIELDS = 94

# node fields that cross the host boundary in the e2e loop
E2E_UP = ["VX", "VY", "PR", "SXX", "SXY", "EXX", "EXY", "ESP"]
E2E_DOWN = ["NU_M2C", "GG", "ND_M2C", "GD", "RO", "MRX", "MRY", "MVX", "MVY", "SPPE",
            "SXXE", "SXYE", "EXXE", "EXYE", "PHIS", "TK"]


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ helpers
def max_over_ranks(x: float, dist, device) -> float:
    """Largest x over the ranks of the job (x itself when not distributed).
    The step time of N replicas is the slowest replica's."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(markers_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job markers/s: every rank steps its own replica of the workload."""
    return world * markers_per_rank / (ms_max * 1e-3)


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(kernel: str):
    """DRAM bytes per marker of `kernel` from the committed ncu summary
    (profiles/traffic.json, one ncu pass at C4); the caller scales it by
    the markers of a launch."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get(kernel)
    return None


def cpu_baseline(steps: int = 3, warmup: int = 1, threads: int | None = None) -> dict:
    """Reference routines (oracle/_ref, compiled from the reference sources
    with floating-point contraction allowed, as the reference's own build
    does) on a window of the same workload, all host cores, plus the same
    routines on one thread (one warm-up and one timed step).  The window is
    1001 x 401 grid lines of the C4 configuration (8 M markers, the slab and
    the frictional band inside it): its node arrays (~0.5 GB) are far beyond
    the host's caches, as the full configuration's are."""
    import oracle
    from oracle import bindings as B
    from velo2cycles_gb300 import synth

    oracle.build()
    threads = threads or os.cpu_count() or 1
    case = synth.make_case("c4", seed=1, window=(1200, 0, 1001, 401))
    one = None
    if B.reference_available():
        res = B.run_reference(case, nthreads=threads, nsteps=steps, warmup=warmup, fast=True)
        secs = float(res["seconds"][:6].sum()) / steps
        kind = "reference"
        r1 = B.run_reference(case, nthreads=1, nsteps=1, warmup=1, fast=True)
        one = case.n / float(r1["seconds"][:6].sum())
    else:
        r = oracle.Restatement(case.copy())
        for _ in range(warmup):
            r.step()
        t = time.perf_counter()
        for _ in range(steps):
            r.step()
        secs = (time.perf_counter() - t) / steps
        threads, kind = 1, "port"
    return {"value": case.n / secs, "unit": UNIT, "cores": threads, "kind": kind,
            "value_1thread": one,
            "sample": f"c4 window of 1001x401 grid lines at the c4 spacing, {case.n} markers, "
                      f"{warmup} warm-up + {steps} timed steps, full MIC step, "
                      "FP contraction allowed",
            "seconds_per_step": secs}


def reference_full(args, threads: int | None = None) -> dict:
    """The reference's routines (oracle/_ref/v2c_ref_full: contraction
    allowed, arrays sized for the full C4 configuration) on the GPU arm's
    own workload -- the same configuration, seed and time step -- with all
    host cores: W warm-up and K timed steps of the full MIC step, the
    per-stage seconds only coming back."""
    import oracle
    from oracle import bindings as B
    from velo2cycles_gb300 import synth

    oracle.build()
    if not os.path.exists(B.reference_path(full=True)):
        raise RuntimeError("full-size reference build unavailable")
    import gc
    import subprocess
    import tempfile

    threads = threads or os.cpu_count() or 1
    case = synth.make_case(args.config, seed=1, interpolationmod=args.interpolationmod)
    n, xn, yn = case.n, case.params["xnumx"], case.params["ynumy"]
    with tempfile.TemporaryDirectory(dir=B.scratch_dir(case)) as d:
        cp, rp = os.path.join(d, "case.bin"), os.path.join(d, "res.bin")
        B.write_case(cp, case, B.ALL_STAGES | B.TIMING_ONLY, threads, args.steps, args.warmup)
        del case  # the reference process holds its own copy (~20 GB at C4)
        gc.collect()
        r = subprocess.run([B.reference_path(full=True), cp, rp], cwd=d, capture_output=True,
                           env=dict(os.environ, OMP_NUM_THREADS=str(threads)),
                           preexec_fn=B.big_stack, timeout=3600)
        if r.returncode != 0:
            raise RuntimeError(f"v2c_ref_full failed ({r.returncode}): "
                               f"{r.stderr.decode()[-500:]}")
        res = B.read_result(rp, 0)
    secs = float(res["seconds"][:6].sum()) / args.steps
    return {"value": n / secs, "unit": UNIT, "cores": threads, "kind": "reference",
            "value_1thread": None,
            "sample": f"the full {args.config} workload ({xn}x{yn} grid lines, {n} markers), "
                      f"{args.warmup} warm-up + {args.steps} timed steps, full MIC step, "
                      "FP contraction allowed",
            "seconds_per_step": secs, "same_config": True}


# ------------------------------------------------------- reference arm
def run_reference_arm(args, rank: int) -> None:
    if rank != 0:
        return
    try:
        base = reference_full(args)
    except Exception as e:  # no full-size build or not enough host memory: the window
        log(f"[bench] reference on the full workload unavailable ({e}); timing the window")
        base = dict(cpu_baseline(steps=args.steps, warmup=args.warmup), same_config=False)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": base["seconds_per_step"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": (f"{args.config} marker-in-cell step, full workload"
                                if base["same_config"] else
                                "c4 marker-in-cell step (bounded window, see cpu_baseline.sample)")},
        "same_config": base["same_config"],
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample",
                                              "value_1thread")},
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU arm
# Newton forms timed on the same steps: (name, start guess, arithmetic)
MODES = [("learned_split", "GUESS_LEARNED", "NEWTON_SPLIT"),
         ("plain_split", "GUESS_PLAIN", "NEWTON_SPLIT"),
         ("plain_fp64", "GUESS_PLAIN", "NEWTON_FP64"),
         ("learned_fp64", "GUESS_LEARNED", "NEWTON_FP64")]
# not timed by default: the step with the per-marker Newton switched off
EXTRA_FORMS = [("no_newton", "GUESS_OFF", "NEWTON_SPLIT")]


def dt_sequence(k: int, seed: int) -> np.ndarray:
    """Per-step time steps, log-uniform in [1e-3, 1e10] s (the coseismic to
    interseismic range of the seismic-cycle runs): each step's slip rates
    differ from the previous step's, so the previous slip rate is not
    already the answer."""
    return 10.0 ** np.random.default_rng(seed).uniform(-3, 10, k)


def train_start_network(m, newton, abi, n_train: int, seed: int) -> dict:
    """Train the start network on the model's own Newton problems, collected
    at 8 time steps, with targets from the plain FP64 solve."""
    import torch
    t0 = time.time()
    per = max(1, n_train // 8)
    stride = max(1, m.n // per)
    dts = dt_sequence(8, seed)
    parts = []
    for dt in dts:
        m.set_params(timestep=float(dt))
        parts.append(newton.collect_states(m, stride=stride))
    S = torch.cat(parts, 1).contiguous()
    m.set_params(newton_precision=abi.NEWTON_FP64)
    out, it = newton.solve(m, S, abi.GUESS_PLAIN, on_device=True)
    T = torch.stack([out[abi.RO_V], out[abi.RO_PHI]]).contiguous()
    loss = newton.train(m, S, T, epochs=4, batch=8192, lr=3e-3, seed=seed)
    torch.cuda.synchronize()
    return {"states": int(S.shape[1]), "loss": float(loss), "seconds": time.time() - t0}


def newton_c3(m, newton, abi, n: int = 4_000_000) -> dict:
    """Per-marker Newton alone on n seeded states (the C3 benchmark), each
    form timed with CUDA events; the network is retrained on these states'
    plain FP64 solutions first."""
    import torch
    S = torch.from_numpy(newton.rsf_states(n, seed=101)).cuda()
    m.set_params(newton_precision=abi.NEWTON_FP64)
    out, _ = newton.solve(m, S, abi.GUESS_PLAIN, on_device=True)
    T = torch.stack([out[abi.RO_V], out[abi.RO_PHI]]).contiguous()
    newton.train(m, S, T, epochs=4, batch=8192, lr=3e-3, seed=3)
    res = {}
    for name, guess, prec in MODES:
        m.set_params(newton_precision=getattr(abi, prec))
        newton.solve(m, S, getattr(abi, guess), on_device=True)
        torch.cuda.synchronize()
        best, its = None, None
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            o, it = newton.solve(m, S, getattr(abi, guess), on_device=True)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            if best is None or ms < best:
                best, its = ms, it
        o = o.cpu().numpy()
        res[name] = {"ms": best, "states_per_s": n / (best * 1e-3),
                     "iters_per_state": float(its.abs().double().mean().item()),
                     "max_residual": float(o[abi.RO_RES].max()),
                     "nonconverged": int((its < 0).sum().item())}
    res["states"] = n
    return res


def run_gpu(args, rank: int, world: int) -> None:
    import torch

    from velo2cycles_gb300 import abi, build, mic, newton, synth

    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    t0 = time.time()
    window = tuple(int(v) for v in args.window.split(",")) if args.window else None
    case = synth.make_case(args.config, seed=1 + rank, interpolationmod=args.interpolationmod,
                           window=window)
    log(f"[bench] {args.config}: {case.n} markers, {case.nodenum} nodes, generated in "
        f"{time.time() - t0:.1f}s")
    stream = torch.cuda.Stream()
    m = mic.MarkerInCell(case.params, case.n, stream=stream.cuda_stream)
    m.set_grid(case.gx, case.gy)
    m.set_rock_table(case.rt)
    m.set_bonds(case.bondm, case.bondn, case.bondv)
    m.upload_markers(case.marks, case.markt)
    m.upload_nodes(case.nodes)
    m.synchronize()
    n = case.n
    log(f"[bench] uploaded in {time.time() - t0:.1f}s")
    forms = [f for f in MODES + EXTRA_FORMS if f[0] in args.forms.split(",")]
    if not forms or forms[0][0] != "learned_split":
        raise SystemExit("--forms must start with learned_split (the headline form)")
    training = None
    if any(g == "GUESS_LEARNED" for _, g, _ in forms):
        training = train_start_network(m, newton, abi, 4_000_000, seed=11)
        log(f"[bench] start network trained: {training}")
    dts = dt_sequence(args.warmup + args.steps, seed=7)

    def step(dt):
        m.set_params(timestep=float(dt))
        m.marker2nodes()
        m.interpolate_center2basic_old()
        m.compute_before_solve(dt, 0)
        m.compute_after_solve(dt, 0)
        m.nodes2markers_move()

    def run_mode(guess, prec, timed_clock=None):
        # every form starts from the same uploaded state
        m.upload_markers(case.marks, case.markt)
        m.upload_nodes(case.nodes)
        m.set_params(newton_guess=getattr(abi, guess), newton_precision=getattr(abi, prec))
        for k in range(args.warmup):
            step(dts[k])
        m.synchronize()
        if timed_clock:
            timed_clock.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        st0 = m.status()
        m.set_profiling(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            step(dts[args.warmup + k])
        e1.record(stream)
        torch.cuda.synchronize()
        st1 = m.status()
        prof = m.profile()
        m.set_profiling(False)
        if dist:
            dist.barrier()
        ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist, "cuda")
        return {
            "ms_per_step": ms, "markers_per_s": replica_throughput(n, world, ms),
            "newton_iters_per_marker": (st1["newton_iters"] - st0["newton_iters"]) / (n * args.steps),
            "newton_fallbacks": st1["newton_fallbacks"] - st0["newton_fallbacks"],
            "newton_nonconverged": st1["newton_nonconv"] - st0["newton_nonconv"],
            "newton_max_residual": st1["newton_max_res"],
            "stage_ms": {k: v[0] / args.steps for k, v in prof.items() if v[1] > 0},
            "launches": int(st1["kernel_launches"] - st0["kernel_launches"]),
        }

    # end to end through the C ABI with host node buffers, learned split form
    nn = case.nodenum
    up = {getattr(abi, "NF_" + f): torch.from_numpy(case.nodes[getattr(abi, "NF_" + f)]).pin_memory().numpy()
          for f in E2E_UP}
    down = {getattr(abi, "NF_" + f): torch.empty(nn, dtype=torch.float64, pin_memory=True).numpy()
            for f in E2E_DOWN}
    import ctypes

    from velo2cycles_gb300._lib import call

    dp = ctypes.POINTER(ctypes.c_double)
    down_f = (ctypes.c_int * len(down))(*down.keys())
    down_p = (dp * len(down))(*[a.ctypes.data_as(dp) for a in down.values()])
    up_f = (ctypes.c_int * len(up))(*up.keys())
    up_p = (dp * len(up))(*[a.ctypes.data_as(dp) for a in up.values()])

    def e2e_step(dt):
        m.set_params(timestep=float(dt))
        m.marker2nodes()
        # the Stokes and temperature inputs leave under the node kernels;
        # the host solver would start reading them at the wait
        call("v2c_download_node_fields_async", m.h, len(down), down_f, down_p)
        m.interpolate_center2basic_old()
        m.compute_before_solve(dt, 0)
        m.compute_after_solve(dt, 0)
        call("v2c_wait_downloads", m.h)
        call("v2c_upload_node_fields", m.h, len(up), up_f, up_p)
        m.nodes2markers_move()

    def run_e2e():
        m.upload_markers(case.marks, case.markt)
        m.upload_nodes(case.nodes)
        m.set_params(newton_guess=abi.GUESS_LEARNED, newton_precision=abi.NEWTON_SPLIT)
        for k in range(max(1, args.warmup)):
            e2e_step(dts[k])
        m.synchronize()
        s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s2.record(stream)
        for k in range(args.steps):
            e2e_step(dts[args.warmup + k])
        e2.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(s2.elapsed_time(e2) / args.steps, dist, "cuda")

    modes = {}
    ms_e2e = None
    clocks = ClockSampler(local)
    for name, guess, prec in forms:
        modes[name] = run_mode(guess, prec, clocks if name == "learned_split" else None)
        if name == "learned_split":
            clk = clocks.stop()
            # the end-to-end loop right after the headline form, on the same
            # warm state of the GPU
            if not args.no_e2e:
                ms_e2e = run_e2e()
                log(f"[bench] e2e: {ms_e2e:.2f} ms/step")
        log(f"[bench] {name}: {modes[name]['ms_per_step']:.2f} ms/step")
    head = modes["learned_split"]
    ms, value, stage_ms = head["ms_per_step"], head["markers_per_s"], head["stage_ms"]

    c3 = newton_c3(m, newton, abi) if rank == 0 and not args.no_c3 else None

    if rank != 0:
        m.close()
        if dist:
            dist.destroy_process_group()
        return

    # roofline of the dominant HBM-streaming kernel (the scatter and the
    # gather/move sweeps; the per-marker physics + Newton is compute-bound)
    peaks = measured_peaks()
    mpn = n / nn
    dom = max(("m2n", "n2m", "move"), key=lambda k: stage_ms.get(k, 0.0))
    alg = n * (ALG_BYTES[dom] + NODE_FIELDS[dom] * 4 / mpn)
    achieved = alg / (stage_ms[dom] * 1e-3) / 1e9
    tr = ncu_traffic(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
            "traffic": (tr * n) if tr is not None else None,
            "peak_source": peaks["source"],
            "alg_bytes_per_marker": ALG_BYTES[dom] + NODE_FIELDS[dom] * 4 / mpn}
    step_alg = STEP_MARKER_BYTES + STEP_NODE_FIELDS * 4 / mpn
    base = cpu_baseline() if not args.no_cpu_baseline else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 fields, f64 node normalisation", "data": "synthetic",
        "config": {"workload": f"{args.config}{' window ' + args.window if args.window else ''}: "
                               f"{case.params['xnumx']}x{case.params['ynumy']} grid, "
                               f"{n} markers ({mpn:.1f}/node), RK4, "
                               f"interpolationmod={args.interpolationmod}, "
                               "antidiffinter=1, per-marker VEP+RSF Newton to 1e-10, learned "
                               "start, split precision",
                   "dt": "per step log-uniform [1e-3, 1e10] s, seeded, same sequence for every form",
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas only"},
        "stage_ms": stage_ms,
        "newton_forms": modes,
        "learned_split_vs_plain_fp64": (modes["plain_fp64"]["ms_per_step"] / ms
                                        if "plain_fp64" in modes else None),
        "learned_split_vs_plain_split": (modes["plain_split"]["ms_per_step"] / ms
                                         if "plain_split" in modes else None),
        "start_network": training,
        "newton_c3": c3,
        "step_alg_bytes_per_marker": step_alg,
        "step_roofline_frac": (value / world) * step_alg / (peaks["hbm_gbs"] * 1e9),
        "roofline": roof,
        "cpu_baseline": ({k: base[k] for k in ("value", "unit", "cores", "kind", "sample",
                                               "value_1thread")}
                         if base else None),
        "e2e": ({"value": replica_throughput(n, world, ms_e2e), "unit": UNIT,
                 "h2d_bytes_per_step": 8 * nn * len(E2E_UP),
                 "d2h_bytes_per_step": 8 * nn * len(E2E_DOWN)} if ms_e2e else None),
        "gpu_launches": head["launches"],
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    m.close()
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------- seismic cycle (C5)
class _OracleCycle:
    """The cycle step on the oracle restatement (FP64): the reference's own
    algorithm, for the drift figures of the GPU reference form."""

    def __init__(self, case, fields):
        import oracle
        self.r = oracle.Restatement(case.copy())
        self.fields = fields
        self.timesum = float(case.params["timesum"])
        self.slip = np.zeros(case.nodenum)
        yn = case.gy.size
        m = np.arange(case.nodenum)
        self.inner = ((m // yn >= 1) & (m % yn >= 1) & (m // yn < case.gx.size - 1) &
                      (m % yn < yn - 1))

    def cycle_step(self, regime, dt):
        from velo2cycles_gb300 import abi
        r = self.r
        r.nodes[abi.NF_VX][:] = self.fields[regime][0]
        r.nodes[abi.NF_VY][:] = self.fields[regime][1]
        r.set_params(timestep=dt, timesum=self.timesum)
        r.marker2nodes(); r.center2basic_old(); r.compute_before_solve(dt, 0); r.basic2center()
        r.recompute_stress(dt); r.center2basic(dt); r.compute_after_solve(dt, 0); r.copyarrays()
        self.slip[self.inner] += dt * r.nodes[abi.NF_RK_SLIPRS_FINAL][self.inner]
        r.nodes2markers(); r.move()
        self.timesum += dt
        r.set_params(timesum=self.timesum)

    def calc_timestep(self, oldornew):
        return self.r.calc_timestep(oldornew)[1]


class _GpuCycle:
    def __init__(self, m, graph):
        self.m, self.graph = m, graph

    def cycle_step(self, regime, dt):
        self.m.cycle_step(regime, dt, use_graph=self.graph)

    def calc_timestep(self, oldornew):
        return self.m.calc_timestep(oldornew)


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    fin = np.isfinite(b) & np.isfinite(a)
    s = np.abs(b[fin]).max() if fin.any() else 0.0
    return float(np.abs(a[fin] - b[fin]).max() / s) if s > 0 else 0.0


def _drift(a, b) -> dict:
    """|a - b| over the finite entries relative to the RMS of b: the bulk
    (rms), the tail (p99) and the worst entry (max)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    fin = np.isfinite(a) & np.isfinite(b)
    d = np.abs(a[fin] - b[fin])
    s = float(np.sqrt(np.mean(b[fin] ** 2))) if fin.any() else 0.0
    if s == 0.0 or not d.size:
        return {"rms": 0.0, "p99": 0.0, "max": 0.0}
    return {"rms": float(np.sqrt(np.mean(d ** 2)) / s), "p99": float(np.quantile(d, 0.99) / s),
            "max": float(d.max() / s)}


def run_cycle(args) -> None:
    """Config 5: the seismic-cycle step sequence on the C1 geometry (480 k
    markers), per-regime CUDA graphs.  The plain FP64 form decides the regime
    and dt sequence; the learned split form replays it (and its own decisions
    are compared); graph and eager replays are timed; the reference form (no
    per-marker Newton) is compared with the FP64 oracle over one compressed
    event."""
    import torch
    from velo2cycles_gb300 import abi, cycle, mic, newton, synth
    steps = args.cycle_steps
    case = synth.make_case("c1", seed=1)
    sched = cycle.Schedule()
    fields = cycle.pulse_fields(case, sched)

    def ctx(**kw):
        c = case.copy()
        c.params.update(kw)
        m = mic.from_case(c)
        for k in (0, 1):
            m.cycle_set_velocity(k, *fields[k])
        return m

    out = {"metric": "seismic-cycle step sequence (config 5)", "unit": "markers/s",
           "config": {"workload": f"c1 geometry, {case.n} markers, {steps} steps, dt "
                                  f"{sched.dt_inter:g} s / {sched.dt_co:g} s on the slip rate, "
                                  f"events every {sched.n_inter} interseismic steps, "
                                  f"{sched.v_pulse:g} m/s pulse for {sched.slip_budget:g} m"},
           "stand_in": "prescribed velocities (load field, load + slip pulse) replace the "
                       "host Stokes solve"}
    forms = {}
    seq = None
    for name, guess, prec in (("plain_fp64", abi.GUESS_PLAIN, abi.NEWTON_FP64),
                              ("learned_split", abi.GUESS_LEARNED, abi.NEWTON_SPLIT)):
        m = ctx(newton_guess=guess, newton_precision=prec)
        if guess == abi.GUESS_LEARNED:
            train_start_network(m, newton, abi, 1_000_000, seed=3)
            m.upload_markers(case.marks, case.markt)
            m.upload_nodes(case.nodes)
            m.set_params(newton_guess=guess, newton_precision=prec,
                         **{k: case.params[k] for k in ("timesum", "timestep")})
            for k in (0, 1):
                m.cycle_set_velocity(k, *fields[k])
        st0 = m.status()
        torch.cuda.synchronize()
        rec = cycle.run(_GpuCycle(m, True), sched, steps, forced=seq)
        st1 = m.status()
        if seq is None:
            seq = list(zip(rec.regime, rec.dt))
        drv = cycle.Driver(sched)
        own = [(0, sched.dt_inter)] + [drv.next(v) for v in rec.maxvel[:-1]]
        forms[name] = {
            "seconds": rec.seconds, "markers_per_s": case.n * steps / rec.seconds,
            "newton_iters_per_marker": (st1["newton_iters"] - st0["newton_iters"]) / (case.n * steps),
            "newton_nonconverged": st1["newton_nonconv"] - st0["newton_nonconv"],
            "newton_max_res": st1["newton_max_res"],
            "coseismic_steps": int(sum(r == 1 for r in rec.regime)),
            "dt_co_steps": int(sum(d == sched.dt_co for d in rec.dt)),
            "own_decisions_differ": int(sum(a != b for a, b in zip(own, seq))),
            "events": int(sum(1 for a, b in zip(rec.regime[1:], rec.regime[:-1]) if a == 1 and b == 0)),
            "max_slip_rate": max(rec.maxvel),
            "_slip": m.cycle_slip(), "_mslip": m.cycle_marker_slip(),
            "_slipv": m.download_markers([abi.MF_SLIPV])[abi.MF_SLIPV],
        }
        m.close()
    p, l = forms["plain_fp64"], forms["learned_split"]
    # the per-marker Newton writes only the marker slip rate, which the
    # reference's own path does not read: node fields, stresses and positions
    # of the two forms are identical (the node slip below checks it), and
    # their difference is the Newton's
    out["drift_learned_split_vs_plain_fp64"] = {
        "node_slip_max": _rel(l["_slip"], p["_slip"]),
        "marker_accumulated_slip": _drift(l["_mslip"], p["_mslip"]),
        "marker_slip_rate_last_step": _drift(l["_slipv"], p["_slipv"])}
    for f in forms.values():
        for k in ("_slip", "_mslip", "_slipv"):
            f.pop(k)
    out["forms"] = forms
    out["value"] = l["markers_per_s"]
    # graph against eager launches on the same sequence (learned split)
    timing = {}
    for graph in (True, False):
        m = ctx(newton_guess=abi.GUESS_PLAIN, newton_precision=abi.NEWTON_SPLIT)
        n = max(1, min(steps - 20, 400))
        cycle.run(_GpuCycle(m, graph), sched, 20, forced=seq[:20])
        rec = cycle.run(_GpuCycle(m, graph), sched, n, forced=seq[20:20 + n])
        timing["graph" if graph else "eager"] = {"steps": n, "seconds": rec.seconds,
                                                 "markers_per_s": case.n * n / rec.seconds}
        m.close()
    out["graph_vs_eager_plain_split"] = timing
    # the reference form against the FP64 oracle over one compressed event
    if args.cycle_oracle_steps > 0:
        import oracle
        oracle.build()
        k = args.cycle_oracle_steps
        s2 = cycle.Schedule(n_inter=k // 3, slip_budget=sched.dt_co * k / 3)
        ref = _OracleCycle(case, fields)
        t0 = time.perf_counter()
        rec_ref = cycle.run(ref, s2, k)
        t_ref = time.perf_counter() - t0
        m = ctx(newton_guess=abi.GUESS_OFF)
        rec = cycle.run(_GpuCycle(m, True), s2, k, forced=list(zip(rec_ref.regime, rec_ref.dt)))
        mk = m.download_markers([abi.MF_X, abi.MF_XY])
        wx = np.diff(case.gx)[np.clip(np.searchsorted(case.gx, ref.r.marks[abi.MF_X], "right") - 1,
                                      0, case.gx.size - 2)]
        out["drift_reference_form_vs_fp64_oracle"] = {
            "steps": k, "coseismic_steps": int(sum(r == 1 for r in rec_ref.regime)),
            "statistic": "|gpu - oracle| over the entries relative to the RMS of the oracle field",
            "accumulated_slip": _drift(m.cycle_slip()[ref.inner], ref.slip[ref.inner]),
            "node_sxy": _drift(m.download_nodes([abi.NF_SXY])[abi.NF_SXY], ref.r.nodes[abi.NF_SXY]),
            "marker_sxy": _drift(mk[abi.MF_XY], ref.r.marks[abi.MF_XY]),
            "marker_x_cells": float((np.abs(mk[abi.MF_X] - ref.r.marks[abi.MF_X]) / wx).max()),
            "oracle_seconds": t_ref, "gpu_seconds": rec.seconds}
        m.close()
        # the sensitivity of the sequence itself: the FP64 oracle from the
        # same state with its marker fields rounded to FP32 (what the device
        # stores at upload; positions kept) and from the state scaled by
        # 1 + 1e-12, same regime and dt sequence
        seq_ref = list(zip(rec_ref.regime, rec_ref.dt))
        sens = {}
        for name, rel in (("fp32_rounded_marker_fields", None), ("relative_1e-12", 1e-12)):
            c = case.copy()
            for f in c.marks:
                if f not in (abi.MF_X, abi.MF_Y):
                    c.marks[f] = (c.marks[f].astype(np.float32).astype(np.float64) if rel is None
                                  else c.marks[f] * (1.0 + rel))
            o2 = _OracleCycle(c, fields)
            cycle.run(o2, s2, k, forced=seq_ref)
            sens[name] = {"accumulated_slip": _drift(o2.slip[o2.inner], ref.slip[ref.inner]),
                          "node_sxy": _drift(o2.r.nodes[abi.NF_SXY], ref.r.nodes[abi.NF_SXY]),
                          "marker_sxy": _drift(o2.r.marks[abi.MF_XY], ref.r.marks[abi.MF_XY])}
        out["drift_fp64_oracle_from_perturbed_state"] = sens
    print(json.dumps(out), flush=True)


def run_stokes(args) -> None:
    """The Stokes matrix assembly (preparematrix + gausmat4_add) on the C2
    grid (1001 x 401 lines, 1.2 M equations) from the node fields of one
    marker2nodes / compute_before_solve / basic2center pass: device time
    (count, scan and fill kernels, CUDA events), the call end to end (CSR
    arrays copied to host memory), the arrays against the oracle
    restatement on the same node values (bit for bit), and the reference's
    own preparematrix on the same values (one host thread; it has no
    OpenMP)."""
    from oracle import bindings as B
    import oracle
    from velo2cycles_gb300 import abi, mic, synth
    oracle.build()
    case = synth.make_case("c2", seed=2)
    dt = float(case.params["timestep"])
    m = mic.from_case(case)
    m.marker2nodes()
    m.compute_before_solve(dt, 0)
    m.interpolate_basic2center()
    ctl = dict(abi.STOKES_DEFAULTS, mukoef=dt * 30e5, dt=dt)
    got = m.stokes_assemble(**ctl)
    rows, nnz = got["b"].size, got["ja"].size
    c = abi.StokesCtl(**ctl)
    P = ctypes.POINTER
    ia, ja = np.zeros(rows + 1, dtype=np.int32), np.zeros(nnz, dtype=np.int32)
    a, b = np.zeros(nnz), np.zeros(rows)
    n_out = ctypes.c_long(0)
    ptrs = (ia.ctypes.data_as(P(ctypes.c_int)), ja.ctypes.data_as(P(ctypes.c_int)),
            a.ctypes.data_as(P(ctypes.c_double)), b.ctypes.data_as(P(ctypes.c_double)))
    from velo2cycles_gb300._lib import call
    for _ in range(args.warmup):
        call("v2c_stokes_assemble", m.h, ctypes.byref(c), nnz, *ptrs, ctypes.byref(n_out))
    m.set_profiling(True)
    p0 = m.profile()["stokes"]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call("v2c_stokes_assemble", m.h, ctypes.byref(c), nnz, *ptrs, ctypes.byref(n_out))
    t_e2e = (time.perf_counter() - t0) / args.steps
    p1 = m.profile()["stokes"]
    dev_ms = (p1[0] - p0[0]) / args.steps
    # the same node values as FP64 for the restatement and the reference
    cc = case.copy()
    nodes = m.download_nodes(list(range(abi.NF_N)))
    for f in range(abi.NF_N):
        cc.nodes[f] = nodes[f]
    t0 = time.perf_counter()
    rc, ref = oracle.Restatement(cc.copy()).stokes_assemble(**ctl)
    t_port = time.perf_counter() - t0
    same = rc == 0 and all(np.array_equal(got[k], ref[k], equal_nan=k in ("a", "b"))
                           for k in ("ia", "ja", "a", "b"))
    t_ref = None
    if B.reference_available():
        t_ref = B.run_reference(cc, stages=B.STOKES_STAGE, stokes=ctl)["stokes"]["seconds"]
    out_bytes = nnz * 12 + rows * 12
    print(json.dumps({
        "metric": "Stokes assembly (preparematrix) equations/s", "unit": "equations/s",
        "value": rows / (dev_ms * 1e-3), "config": {"workload": f"c2 grid, {rows} equations, "
                                                                f"{nnz} coefficients"},
        "device_ms": dev_ms, "e2e": {"value": rows / t_e2e, "unit": "equations/s",
                                     "ms": t_e2e * 1e3, "d2h_bytes": out_bytes},
        "csr_output_gbs_device": out_bytes / (dev_ms * 1e-3) / 1e9,
        "bit_exact_vs_oracle": bool(same),
        "cpu_oracle_port_1thread": {"value": rows / t_port, "seconds": t_port},
        "cpu_reference_1thread": ({"value": rows / t_ref, "seconds": t_ref} if t_ref else None),
    }), flush=True)
    m.close()


def run_c2_parity(args) -> None:
    """Config 2: the reference form (per-marker Newton off) on the C2 grid
    (non-uniform, 1001 x 401 lines, 6.4 M markers) for K steps with dt
    log-uniform in [1e-3, 1e10] s, against the reference's own routines
    (compiled from its sources, all host threads) on the same sequence:
    per-field error after the last step."""
    from oracle import bindings as B
    import oracle
    from velo2cycles_gb300 import abi, mic, synth
    oracle.build()
    if not B.reference_available():
        print(json.dumps({"c2_parity": "unavailable: the reference routines are not built"}))
        return
    k = args.c2_steps
    case = synth.make_case("c2", seed=2)
    dts = dt_sequence(k, seed=7)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = B.run_reference(case, nthreads=threads, nsteps=k, dts=dts)
    t_ref = time.perf_counter() - t0
    c = case.copy()
    c.params.update(newton_guess=abi.GUESS_OFF)
    m = mic.from_case(c)
    ts = float(case.params["timesum"])
    t0 = time.perf_counter()
    for dt in dts:
        m.set_params(timestep=float(dt), timesum=ts)
        m.step()
        ts += float(dt)
    m.synchronize()
    t_gpu = time.perf_counter() - t0
    nodes = m.download_nodes()
    marks = m.download_markers()
    names_n, names_m = abi.node_field_names(), abi.marker_field_names()
    per_node, per_mark = {}, {}
    for f in range(abi.NF_N):
        if np.array_equal(ref["nodes"][f], case.nodes[f]) and np.array_equal(nodes[f], case.nodes[f]):
            continue  # not written by the step
        per_node[names_n[f]] = {"max_rel": _rel(nodes[f], ref["nodes"][f]),
                                **_drift(nodes[f], ref["nodes"][f])}
    kept = (abi.MF_X, abi.MF_Y, abi.MF_K, abi.MF_E, abi.MF_P, abi.MF_XX, abi.MF_XY, abi.MF_EXX,
            abi.MF_EXY, abi.MF_VX, abi.MF_VY, abi.MF_PHI, abi.MF_C)
    for f in kept:  # the marker fields the device keeps
        per_mark[names_m[f]] = {"max_rel": _rel(marks[f], ref["marks"][f]),
                                **_drift(marks[f], ref["marks"][f])}
    gx = case.gx
    ix = np.clip(np.searchsorted(gx, ref["marks"][abi.MF_X], "right") - 1, 0, gx.size - 2)
    out = {"c2_parity": {"steps": k, "markers": case.n, "reference_threads": threads,
                         "reference_seconds": t_ref, "gpu_seconds": t_gpu,
                         "statistics": "max_rel: max |gpu - ref| / max |ref|; rms, p99, max: "
                                       "relative to the RMS of the reference field",
                         "marker_x_cells": float((np.abs(marks[abi.MF_X] - ref["marks"][abi.MF_X]) /
                                                  np.diff(gx)[ix]).max()),
                         "nodes": per_node, "markers": per_mark}}
    m.close()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c4")
    ap.add_argument("--window", default="",
                    help="i0,j0,nx,ny: a window of nx x ny grid lines of the configuration "
                         "(a small case of the same spacing for profiler captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="skip the Newton-only C3 block")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end loop")
    ap.add_argument("--forms", default=",".join(f[0] for f in MODES),
                    help="Newton forms to time, comma-separated, learned_split first")
    ap.add_argument("--cycle", action="store_true",
                    help="the seismic-cycle step sequence (config 5) instead of the C4 step")
    ap.add_argument("--cycle-steps", type=int, default=1000)
    ap.add_argument("--cycle-oracle-steps", type=int, default=60,
                    help="steps of the reference form against the FP64 oracle (0: skip)")
    ap.add_argument("--c2-parity", action="store_true",
                    help="config 2: per-field error against the reference's routines")
    ap.add_argument("--c2-steps", type=int, default=100)
    ap.add_argument("--interpolationmod", type=int, default=2, choices=[1, 2],
                    help="marker-node stencil: 2 (shipped default) or 1 (13-node)")
    ap.add_argument("--stokes", action="store_true",
                    help="the Stokes matrix assembly on the C2 grid")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
    elif args.cycle:
        if rank == 0:
            run_cycle(args)
    elif args.c2_parity:
        if rank == 0:
            run_c2_parity(args)
    elif args.stokes:
        if rank == 0:
            run_stokes(args)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
