#!/usr/bin/env python3
"""Throughput of the sea-ice dynamics step on GB300: cell-updates per second.

Workload (the configuration the headline metric is quoted on, one GPU): the
512 x 512 box test with DG2 transport (6 components), CG2 velocity, DG-stress
8, 100 mEVP iterations (alpha = beta = 300) per 120 s step, in the mixed
precision mode (FP32 stress/momentum arithmetic and state; FP64 for the
conservation sums, the inverse mass matrices, Delta and the viscosity).
One "step" is one model step: the DG transport of concentration and
thickness with limiters, the preparation of the momentum solve and the 100
mEVP iterations (strain, stress, divergence, momentum, boundaries).

  value  device-resident: K steps of the CUDA graph, CUDA events on the
         library's stream; not re-flushed between steps: each step sweeps
         more than L2 holds (the FP32 transport operators, the FP64 inverse
         mass matrices and stage buffers, the sub-cycle's working set).
  e2e    the reference's module cycle through the C ABI with host buffers
         (MEVPDynamics::update: setData of h, A, winds, ocean, ssh, then
         update, then getDG0Data of h, A, u, v and the ice-ocean stress),
         13 C-ABI calls per step, wall clock, host<->device copies inside.
         e2e_module_step: the same cycle as one nsdg_kernel_module_step
         call per step (what the GPUMEVPDynamics module makes);
         e2e_pageable / e2e_module_step_pageable: the same with the
         pageable arrays a model holds (moved by a kernel that reads and
         writes them directly where the GPU allows it).
  variants.plain_fp64     the FP64 path (the reference's arithmetic) on the
                          same grid, with its own roofline;
  variants.learned_fp32   the learned warm start as configured for it:
                          data from 2000 plain steps on 256^2 boxes with
                          randomised cyclone tracks, training on the GPU,
                          then the warm update on 1024^2 with and without
                          audit against the plain sub-cycle, and a plain
                          statement of the speed-up at equal error (or none);
  variants.ice_growth     the column thermodynamics before the dynamics
                          (IceGrowth + ThermoIce0 + HiblerSpread +
                          ConstantHealing) on the same cell count;
  velocity_error_vs_fp64  one simulated day: FP32 path vs FP64 path, next to
                          the FP64 path's own response to h x (1 + 1e-14),
                          with the FP64 path at h x (1 + 2e-14) and the FP32
                          path at h x (1 + 1e-14) beside them (which runs the
                          library flags non-finite, and when).

--precision fp64 --nx 256 gives the FP64 drop-in path on the 256^2 grid.
--ensemble 32 times the 32-member uneven ensemble alone.
--table prints one line per benchmark configuration (64^2 DG1, 256^2, 512^2
with BBM, the ensemble, 1024^2): the oracle on all host threads and on one
thread beside the GPU paths.
--day-error bbm|parts prints error checkpoints over a simulated day (the BBM
at 512^2; the parts of the mixed path at 256^2) against the FP64 path.

--impl reference times the CPU restatement of the reference algorithm (the
oracle, pinned against the reference's own code by the golden fixtures) on
the host cores with all threads, on the same workload.  The reference's own
build (oracle/_ref) needs the reference sources, which the timing host does
not have.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "cell-updates/s"
UNIT = "cell-updates/s"
NX = 512
DG = 6
DT = 120.0
ALPHA = BETA = 300.0
NSTEPS = 100


def bytes_per_element_iteration_stress(word: int = 8, spherical: bool = False, parallelogram: bool = False) -> int:
    """Algorithmic DRAM bytes of one launch of the element stress kernel, per
    element: the strain operators G_x, G_y and the divergence operators A_1,
    A_2 (4 x 81 words; on a parallelogram mesh the FP32 kernel reads 5 FP32
    coefficients instead), the pressure terms at the 9 Gauss points (FP64
    P/alpha; in the FP32 kernels FP64 P/(8 alpha) and FP32 P/(2 alpha), the
    latter formed in-kernel by the parallelogram kernel), the
    18 divergence coefficients read and written, and the CG2 velocity counted
    once per node (about 4 nodes per element, u and v)."""
    operators = 5 * 4 if parallelogram else (6 if spherical else 4) * 81 * word  # + G_m, A_3 on a sphere
    # the parallelogram kernel forms P/(2 alpha) from P/(8 alpha) (an exact x4)
    pressure = 9 * 8 + (9 * 4 if word == 4 and not parallelogram else 0)
    tdiv = 2 * 18 * word
    velocity = 4 * 2 * word
    return operators + pressure + tdiv + velocity


def flops_per_element_iteration_stress() -> int:
    """Flops of kMevpStress per element (FMA = 2): strain 4 x 81 FMA, Delta,
    viscosity and stress increments ~12 per Gauss point, divergence update
    4 x 81 FMA + 18."""
    return 2 * (4 * 81) + 9 * 12 + 2 * (4 * 81) + 2 * 18


def bytes_per_cell_update(n_iter: int = NSTEPS, word: int = 8) -> float:
    """Algorithmic bytes per cell-update of the whole step: n_iter x (element
    kernel + node kernel share) + transport/prepare (FP64 in both paths)."""
    node_per_element = 4 * (15 * word) + 18 * word  # ~4 nodes x 15 streams + gathered divergence coefficients
    transport = 4 * (6 * 9 * 2 + 36 + 4 * 6 + 2 * 6) * 8  # cell terms, M^-1, phi, stage I/O
    prepare = 2 * 6 * 8 + 9 * 8 + 20 * 8 * 4
    return n_iter * (bytes_per_element_iteration_stress(word) + node_per_element) + transport + prepare


def transport_bytes_per_element(tiled: bool, word: int = 4, dg: int = 6) -> int:
    """Algorithmic DRAM bytes per element of one step's transport (two RK
    stages of h and A).  Per-element kernel: the cell operators (2 x DG x 9
    words), the FP64 M^{-1} (DG^2), and per field its coefficients, velocity
    share, k1 and output (4 x DG FP64).  Tiled parallelogram kernel: per stage
    the two fields' coefficients, the DG velocity, the diagonal of M^{-1}, the
    four Jacobian coefficients, one X- and one Y-edge's 3 normal velocities,
    and the stage output and k1 (written or read) of both fields."""
    if not tiled:
        return 2 * (2 * dg * 9 * word + dg * dg * 8 + 2 * (4 * dg * 8)) + 4 * 3 * 8
    return 2 * (2 * dg * 8 + 2 * dg * 8 + dg * 8 + 4 * 4 + 2 * 3 * 8 + 2 * (2 * dg * 8))


def launched_bytes_per_cell_update(box, prec: int, stress_kind: str, tiled_transport: bool = False) -> dict:
    """Algorithmic DRAM bytes per cell-update of the kernels one step
    actually launches (each array counted once per launch), by part:
    100 x (element stress kernel + node momentum kernel) + transport,
    preparation and read-outs.  stress_kind names the element kernel:
    "fp64" (FP64 operators), "pairs" (the same bytes as float pairs),
    "affine" (5 FP32 coefficients per element), "tma"/"global" (FP32
    operators)."""
    N = box.nelements
    ncg = (2 * box.nx + 1) * (2 * box.ny + 1)
    word = 8 if prec == 0 else 4
    stress = bytes_per_element_iteration_stress(word, parallelogram=stress_kind == "affine")
    if prec == 0:
        # 15 FP64 node streams read, u and v written, the Dirichlet flag
        node = ncg * (15 * 8 + 2 * 8 + 1) / N
    else:
        # two float4 of per-step constants, u and v read and written (FP32)
        node = ncg * (32 + 4 * 4) / N
    # transport of 2 fields in 2 RK stages: cell operators (FP32 on the mixed
    # path) or the tiled kernel's coefficients, FP64 inverse mass matrices
    # (or their diagonal), phi / k1 / stage I/O, edge velocities
    dg = 6
    transport = transport_bytes_per_element(tiled_transport, word, dg)
    # preparation: CG2DG of u, v, DG2CG of h, A, node and element constants
    prepare = 2 * 9 * 8 + 2 * dg * 8 + 9 * 8 + ncg * (12 * 8) / N
    per_iter = stress + node
    total = NSTEPS * per_iter + transport + prepare
    return {"total": total, "per_iteration_stress": stress, "per_iteration_node_share": node,
            "transport": transport, "prepare": prepare, "stress_kernel": stress_kind,
            "transport_kernel": "tiled" if tiled_transport else "element"}


def transport_record(k, N: int, ms_step: float) -> dict:
    """The transport stage the step uses, timed alone (CUDA events, 50
    launches of one RK stage), beside the per-element kernel on the same
    state, with its algorithmic bandwidth against the measured copy peak."""
    kind, cell_mismatch, offdiag = k.transport_variant()
    tms, tname = k.time_kernel(2, 50)
    ems = k.time_kernel(13, 50)[0]
    bpe = transport_bytes_per_element(kind == "tiled") // 2
    hbm, hbm_kind = measured_peaks()
    ach = N * bpe / (tms * 1e-3) / 1e9
    return {"name": tname, "kernel": kind, "stage_ms": tms, "element_kernel_stage_ms": ems,
            "share_of_step": 2 * tms / ms_step, "algorithmic_bytes_per_element_stage": bpe,
            "achieved_gbs": ach, "peak_gbs": hbm, "frac": ach / hbm, "peak_kind": hbm_kind,
            "cell_operator_mismatch": cell_mismatch, "minv_offdiag": offdiag}


# --------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def fp64_peak_tflops(local: int):
    """FP64 DGEMM throughput (cuBLAS through torch) as the FP64 denominator."""
    try:
        import torch
        dev = torch.device("cuda:0")
        n = 4096
        a = torch.randn(n, n, dtype=torch.float64, device=dev)
        b = torch.randn(n, n, dtype=torch.float64, device=dev)
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize(dev)
        best = 0.0
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize(dev)
            best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        del a, b
        return best, "measured: cuBLAS DGEMM 4096^3 via torch.matmul"
    except Exception as ex:  # torch absent or failing: report the nominal figure
        return 1.25, f"nominal (DGEMM probe failed: {type(ex).__name__})"


# --------------------------------------------------------------------------
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline(nx: int = NX, sample_steps: int = 10, warm: int = 1, single_steps: int = 1):
    """The oracle (CPU restatement of the reference) on the host cores, all
    OpenMP threads, on a bounded sample of the same workload, and the same
    restatement on one thread for `single_steps` steps."""
    from oracle import pyoracle
    from nextsimdg_gb300.boxtest import BoxTest

    pyoracle.load()
    box = BoxTest(nx)
    k = pyoracle.OracleKernel(0, DG, alpha=ALPHA, beta=BETA, n_steps=NSTEPS)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    for s in range(warm):
        k.update(s * DT, DT)
    t0 = time.perf_counter()
    for s in range(sample_steps):
        k.update((warm + s) * DT, DT)
    t = time.perf_counter() - t0
    v = box.nelements * sample_steps / t
    cores = pyoracle.num_threads()
    out = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{sample_steps} model steps of the {nx}x{nx} DG2 box test after {warm} warm-up step(s), "
                     f"{t:.1f} s", "cpu_model": cpu_model()}
    if single_steps > 0:
        pyoracle.set_threads(1)
        try:
            t0 = time.perf_counter()
            for s in range(single_steps):
                k.update((warm + sample_steps + s) * DT, DT)
            t1 = time.perf_counter() - t0
        finally:
            pyoracle.set_threads(cores)
        out["single_thread"] = {"value": box.nelements * single_steps / t1, "unit": UNIT, "cores": 1,
                                "sample": f"{single_steps} model step(s) of the same run, {t1:.1f} s"}
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    from oracle import pyoracle
    from nextsimdg_gb300.boxtest import BoxTest

    pyoracle.load()
    box = BoxTest(args.nx)
    k = pyoracle.OracleKernel(0, DG, alpha=ALPHA, beta=BETA, n_steps=NSTEPS)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    # each step is a full model step of the workload (1.3 s on 16 Arm cores
    # at 512^2): the default 3 + 20 steps finish within a minute
    for s in range(args.warmup):
        k.update(s * DT, DT)
    t0 = time.perf_counter()
    for s in range(args.steps):
        k.update((args.warmup + s) * DT, DT)
    t = time.perf_counter() - t0
    v = box.nelements * args.steps / t
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic box test",
            "config": {"workload": f"box test {args.nx}x{args.nx}, DG2 transport, CG2 velocity, mEVP {NSTEPS} "
                                   f"iterations, alpha=beta={ALPHA:g}, dt={DT:g} s", "precision": "fp64 (oracle)"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": pyoracle.num_threads(), "kind": "port",
                             "sample": f"{args.steps} full model steps after {args.warmup} warm-up"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def make_kernel(box, precision: int, n_steps: int = NSTEPS, scale_h: float = 1.0, alpha: float = ALPHA):
    from nextsimdg_gb300.dynamics import MEVPDynamicsKernel
    k = MEVPDynamicsKernel(dg_comp=DG, alpha=alpha, beta=alpha, n_steps=n_steps, precision=precision)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr * scale_h if name == "hice" else arr)
    return k


def stress_roofline(k, N: int, prec: int, ms_step: float, local: int, nx: int):
    """Roofline of the dominant kernel (the element stress kernel), timed alone
    with CUDA events on the library's stream."""
    kms, kname = k.time_kernel(0, 50)
    nms, nname = k.time_kernel(1, 50)
    kind, mismatch = k.stress_variant()
    affine = kind == "affine"
    bpe = bytes_per_element_iteration_stress(4 if prec else 8, parallelogram=affine)
    achieved = N * bpe / (kms * 1e-3) / 1e9
    hbm, hbm_kind = measured_peaks()
    traffic = None
    prof = ROOT / "profiles" / (f"{kname}_box{nx}_fp32.md" if prec else f"{kname}_box{nx}_fp64.md")
    if prof.exists():
        for line in prof.read_text().splitlines():
            if line.startswith(f"traffic_bytes_per_launch_{nx}:"):
                traffic = int(line.split(":")[1])
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": traffic, "kernel": kname, "kernel_ms": kms, "share_of_step": kms * NSTEPS / ms_step,
            "algorithmic_bytes_per_element": bpe, "peak_kind": hbm_kind,
            "kernel_timing": "CUDA events on the library's stream around 50 back-to-back launches of the kernel "
                             "on the workload's state, right after the timed steps"}
    if prec:
        # every FP32 stress kernel on this mesh: the operator-streaming ones
        # (global loads, TMA tiles) and, on a parallelogram mesh, the
        # coefficient kernel with each FP64 viscosity form
        names = {3: "global", 4: "tma", 5: "affine_rsqrt_f64", 6: "affine_newton_f64", 7: "affine_newton_f64_intcvt",
                 8: "affine_float_pairs", 12: "affine_float_pairs_checked"}
        ids = (3, 4, 5, 6, 7, 8, 12) if affine else (3, 4)
        roof["stress_kernel_ms"] = {names[i]: k.time_kernel(i, 50)[0] for i in ids}
        roof["stress_kernel"] = kind
        roof["parallelogram_mismatch"] = mismatch
        if affine:
            # form 2 (the default: the FP64 Newton step, 3 DFMA + 2 DMUL per
            # Gauss point) is bound by FP64 issue, against the FMA-lane rate
            # of the measured FP64 DGEMM; form 4 computes the same step in
            # float pairs, bitwise equal, and runs the FP64 step only where
            # its rounding check fails (about 1e-4 of the Gauss points)
            form = k.viscosity_form()
            roof["viscosity_form"] = form
            fp64_tf, fp64_kind = fp64_peak_tflops(local)
            inst = N * 9 * 5
            t2 = roof["stress_kernel_ms"]["affine_newton_f64_intcvt"]
            rate = inst / (t2 * 1e-3) / 1e12
            issue = {"kernel_ms": t2, "fp64_instructions_per_launch": inst, "achieved_T_lane_inst_per_s": rate,
                     "peak_T_fma_lanes_per_s": fp64_tf / 2, "frac": rate / (fp64_tf / 2), "peak_kind": fp64_kind}
            if form == 2:
                roof["limiter"] = "fp64 issue (Delta and viscosity in FP64), see fp64_issue"
                roof["fp64_issue"] = issue
            else:
                roof["limiter"] = ("memory and FP32 issue: Delta and the viscosity by float pairs checked against "
                                   "the FP64 form's rounding (bitwise equal); fp64_issue_form2 is the FP64 form")
                roof["fp64_issue_form2"] = issue
    if prec == 0:
        fp64_tf, fp64_kind = fp64_peak_tflops(local)
        ach = N * flops_per_element_iteration_stress() / (kms * 1e-3) / 1e12
        roof["fp64"] = {"achieved_tflops": ach, "peak_tflops": fp64_tf, "frac": ach / fp64_tf,
                        "peak_kind": fp64_kind}
    return roof, {"name": nname, "ms": nms}


def fp64_pairs_variant(args, box, N: int, local: int) -> dict:
    """The FP64 path with the float-pair stress kernel staged by TMA
    (NSDG_FP64_STRESS=pairs_tma): the 9 x 9 operator products, Delta^2 and
    the stress increments in float pairs (about 48 significant bits), 1/Delta
    and the divergence update in FP64; the same operator bytes as FP64."""
    os.environ["NSDG_FP64_STRESS"] = "pairs_tma"
    try:
        k = make_kernel(box, 0)
    finally:
        os.environ.pop("NSDG_FP64_STRESS", None)
    k.time_updates(DT, 3)
    ms = k.time_updates(DT, args.steps) / args.steps
    k.synchronize()
    roof, node = stress_roofline(k, N, 0, ms, local, args.nx)
    times = {name: k.time_kernel(i, 50)[0] for name, i in (("fma", 9), ("pairs_global_loads", 10),
                                                           ("pairs_tma", 11))}
    k.close()
    return {"value": N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "roofline": roof, "node_kernel": node,
            "stress_kernel_ms": times, "stress_kernel": "kMevpStressPairsTma",
            "arithmetic": "operator products, Delta^2 and stress increments in float pairs (about 48 bits); "
                          "1/Delta, P/(8 alpha Delta) and the divergence update in FP64",
            "launched_bytes_per_cell_update": launched_bytes_per_cell_update(box, 0, "pairs")}


def distorted_variant(args, local: int) -> dict:
    """Mixed precision on a 512 x 512 box whose vertices are displaced
    (sinusoidally, 3 % of the box: the elements are general quadrilaterals,
    not parallelograms), so the element kernel streams the per-element FP32
    operators (TMA tiles or global loads, whichever the library times as
    faster on this mesh) instead of the parallelogram coefficients."""
    from nextsimdg_gb300.boxtest import BoxTest
    box = BoxTest(args.nx, distort=0.03)
    N = box.nelements
    k = make_kernel(box, 1)
    k.time_updates(DT, 3)
    ms = k.time_updates(DT, args.steps) / args.steps
    k.synchronize()
    roof, node = stress_roofline(k, N, 1, ms, local, args.nx)
    kind = k.stress_variant()[0]
    transport = transport_record(k, N, ms)
    k.close()
    return {"value": N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "stress_kernel": kind, "roofline": roof,
            "node_kernel": node, "transport_kernel": transport,
            "mesh": "box test vertices displaced by 3 % of the box (sin x sin)",
            "launched_bytes_per_cell_update": launched_bytes_per_cell_update(box, 1, kind)}


def ensemble_variant(args) -> dict:
    """The 32-member uneven ensemble (sides from {64..384}, perturbed
    cyclones and h), batched against the members stepped one by one."""
    r = ensemble_measure(args, 32)
    return {kk: r[kk] for kk in ("value", "unit", "ms_per_step", "cells", "sequential_members", "autotuned_tiles",
                                 "gpu_launches_per_step", "sides", "persistent_subcycle")}


def learned_config5_variant(args) -> dict:
    """The learned warm start as configuration 5 states it: training data from
    2000 plain-solver steps on 256 x 256 box tests with randomised cyclone
    tracks (10 tracks of 200 steps: start within +-50 km of the centre, speed
    8-12 m/s, h noise sigma 0.02 m; every third step a sample), the network
    trained on the GPU, its weights and input normalisation moved unchanged to
    a network of the 1024 x 1024 grid (it is fully convolutional), then the
    1024 x 1024 box test with K mEVP iterations after the network's start
    instead of 100, with the device-side residual fallback.  Speed against the
    plain FP32 step, and the velocity error after `err_steps` steps against
    the plain FP32 sub-cycle (the reference for the warm start's error) and against FP64,
    next to the FP32 path's own error against FP64."""
    from nextsimdg_gb300 import surrogate
    from nextsimdg_gb300.boxtest import BoxTest, step_forcing
    K = args.warm_iters
    rng = np.random.default_rng(7)
    tracks, per_track, stride = 10, 200, 3
    L = 512e3
    net = surrogate.warm_net(256, 256, seed=1)
    capacity = tracks * (per_track // stride)
    net.dataset_reserve(capacity)
    slot, ratios = 0, []
    t0 = time.perf_counter()
    for r in range(tracks):
        tb = BoxTest(256, seed=100 + r, start=(0.5 * L + rng.uniform(-50e3, 50e3), 0.5 * L + rng.uniform(-50e3, 50e3)),
                     wind_speed=float(rng.uniform(8.0, 12.0)), h_noise=0.02)
        kt = make_kernel(tb, 1)
        for st in range(per_track):
            step_forcing(kt, tb, st)
            sl = slot if st % stride == stride - 1 else -1
            ratio = kt.warm_sample(st * DT, DT, K, net, sl)
            if sl >= 0:
                ratios.append(ratio)
                slot += 1
        kt.close()
    net.dataset_normalise(slot)
    loss = float("nan")
    for i, (frac, lr) in enumerate(((0.4, 1e-3), (0.3, 3e-4), (0.3, 1e-4))):
        loss = net.train(slot, max(1, int(args.warm_train_iters * frac)), batch=1, lr=lr, seed=1 + i)
    t_train = time.perf_counter() - t0
    kappa = float(max(ratios))
    big = surrogate.warm_net(1024, 1024, seed=1)
    big.set_params(net.get_params())
    big.set_normalisation(net.get_normalisation())
    net.close()
    box = BoxTest(1024)
    N = box.nelements
    out = {"training": {"grid": "256x256", "tracks": tracks, "plain_steps": tracks * per_track, "samples": slot,
                        "train_iterations": args.warm_train_iters, "train_loss": loss, "data_and_training_s": t_train,
                        "kappa": kappa * 1.5},
           "evaluation_grid": "1024x1024", "k_iters": K}
    plain = make_kernel(box, 1)
    for st in range(args.warmup):
        step_forcing(plain, box, st)
        plain.update(st * DT, DT)
    plain_ms = plain.time_updates(DT, args.steps) / args.steps
    plain.close()
    out["plain_fp32"] = {"value": N / (plain_ms * 1e-3), "ms_per_step": plain_ms}
    for name, je, jt in (("unaudited", 0, 0.0), ("audited_every_10_tol_0.1", 10, 0.1)):
        k = make_kernel(box, 1)
        k.set_warm_start(big, K, kappa * 1.5, je, jt)
        for st in range(args.warmup):
            step_forcing(k, box, st)
            k.update(st * DT, DT)
        ms = k.time_updates(DT, args.steps) / args.steps
        ws = k.warm_stats()
        out[name] = {"value": N / (ms * 1e-3), "ms_per_step": ms, "speedup_vs_plain_fp32": plain_ms / ms,
                     "accepted": ws["accepted"], "fallbacks": ws["fallbacks"], "audited": ws["audited"],
                     "audit_rejected": ws["audit_rejected"], "last_audit_rel_error": ws["last_audit_error"]}
        k.close()
    # error over err_steps steps from the same start: learned (unaudited),
    # plain FP32, FP64
    err_steps = 30
    ks = {"fp64": make_kernel(box, 0), "fp32": make_kernel(box, 1), "learned": make_kernel(box, 1)}
    ks["learned"].set_warm_start(big, K, kappa * 1.5, 0, 0.0)
    for st in range(err_steps):
        for k in ks.values():
            step_forcing(k, box, st)
            k.update(st * DT, DT)
    r = {n: (k.getDG0Data("u"), k.getDG0Data("v")) for n, k in ks.items()}
    rms = lambda a: float(np.sqrt(np.mean(a * a)))  # noqa: E731
    d = lambda a, b: rms(np.hypot(r[a][0] - r[b][0], r[a][1] - r[b][1]))  # noqa: E731
    ws = ks["learned"].warm_stats()
    out["error_after_steps"] = {"steps": err_steps, "learned_vs_plain_fp32_m_per_s": d("learned", "fp32"),
                                "learned_vs_fp64_m_per_s": d("learned", "fp64"),
                                "plain_fp32_vs_fp64_m_per_s": d("fp32", "fp64"),
                                "velocity_rms_m_per_s": rms(np.hypot(*r["fp64"])),
                                "accepted": ws["accepted"], "fallbacks": ws["fallbacks"]}
    for k in ks.values():
        k.close()
    big.close()
    un = out["unaudited"]
    equal = out["error_after_steps"]["learned_vs_plain_fp32_m_per_s"] <= \
        out["error_after_steps"]["plain_fp32_vs_fp64_m_per_s"]
    if un["accepted"] == 0:
        out["speedup_at_equal_error"] = None
        out["statement"] = ("none: the network trained on 256x256 never passes the residual acceptance on "
                            "1024x1024, so every step runs the plain sub-cycle after the network and K "
                            f"iterations ({un['speedup_vs_plain_fp32']:.2f}x the plain FP32 step, same result)")
    elif equal:
        out["speedup_at_equal_error"] = un["speedup_vs_plain_fp32"]
        out["statement"] = (f"{un['speedup_vs_plain_fp32']:.2f}x the plain FP32 step, with the 30-step velocity "
                            "difference to plain FP32 within plain FP32's own difference to FP64")
    else:
        out["speedup_at_equal_error"] = None
        out["statement"] = (f"none at equal error: unaudited {un['speedup_vs_plain_fp32']:.2f}x the plain FP32 "
                            "step, but its 30-step velocity difference to plain FP32 exceeds plain FP32's "
                            "difference to FP64")
    return out


def bbm_variant(args, box, N: int, err_steps: int = 10):
    """The BBM rheology (damage, DG8 stress transport) on the same box with
    damage = 1, FP64 and mixed precision: throughput, and the velocity and
    damage RMS after `err_steps` steps of the FP32 path and of the FP64 path
    with h x (1 + 1e-14), both against the FP64 path."""
    from nextsimdg_gb300._lib import NsdgError
    from nextsimdg_gb300.boxtest import setup_kernel, step_forcing
    from nextsimdg_gb300.dynamics import BBMDynamicsKernel
    # the explicit elastic sub-steps must resolve the elastic wave: dt / n <=
    # dx / (2 sqrt(E / rho)) (813 m/s with the default Young's modulus)
    dx = box.L / box.nx
    sub = max(NSTEPS, int(math.ceil(DT / (0.5 * dx / math.sqrt(5.9467e8 / 900.0)))))
    sub = int(math.ceil(sub / 50.0)) * 50
    out = {"sub_steps": sub, "damage_init": 1.0}
    ks = {}
    for name, prec, scale in (("fp64", 0, 1.0), ("fp64_h_times_1p1e-14", 0, 1.0 + 1e-14), ("fp32", 1, 1.0)):
        k = BBMDynamicsKernel(dg_comp=DG, n_steps=sub, precision=prec)
        k.initialise(box.coords(), False, box.mask())
        for fname, arr in box.initial_fields().items():
            k.setData(fname, arr * scale if fname == "hice" else arr)
        k.setData("damage", box.damage())
        ks[name] = k
    try:
        for s in range(err_steps):
            for k in ks.values():
                step_forcing(k, box, s)
                k.update(s * DT, DT)
        r = {n: {f: k.getDG0Data(f) for f in ("u", "v", "damage", "hice")} for n, k in ks.items()}
        ref = r["fp64"]
        rms = lambda a: float(np.sqrt(np.mean(a * a)))  # noqa: E731
        out["error_vs_fp64"] = {"steps": err_steps}
        for n in ("fp32", "fp64_h_times_1p1e-14"):
            x = r[n]
            out["error_vs_fp64"][n] = {"u_v_rms_m_per_s": rms(np.hypot(x["u"] - ref["u"], x["v"] - ref["v"])),
                                       "damage_rms": rms(x["damage"] - ref["damage"]),
                                       "h_rms_m": rms(x["hice"] - ref["hice"])}
        for name in ("fp64", "fp32"):
            k = ks[name]
            steps = 3
            ms = k.time_updates(DT, steps) / steps
            sms, sname = k.time_kernel(0, 10)
            mms, mname = k.time_kernel(1, 10)
            out[name] = {"value": N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, sname + "_ms": sms,
                         mname + "_ms": mms}
        out["fp32_speedup"] = out["fp64"]["ms_per_step"] / out["fp32"]["ms_per_step"]
    except NsdgError as ex:
        out["error"] = str(ex)
    for k in ks.values():
        k.close()
    return out


def spherical_variant(args, N: int, local: int):
    """The same step on a spherical (lon, lat) mesh of the same size: a
    patch from 57 to 74 degrees north, 34 degrees of longitude, land ring,
    constant thickness and concentration, a spatially varying wind; FP32 and
    FP64.  The FP32 element kernel streams 6 operator blocks instead of 4."""
    from nextsimdg_gb300.dynamics import MEVPDynamicsKernel
    n = args.nx
    lo = np.linspace(-0.3, 0.3, n + 1)
    la = np.linspace(1.0, 1.3, n + 1)
    X, Y = np.meshgrid(lo, la)
    coords = np.stack([X.ravel(), Y.ravel()], 1)
    mask = np.ones((n, n))
    mask[0, :] = mask[-1, :] = 0
    mask[:, 0] = mask[:, -1] = 0
    cx, cy = np.meshgrid(0.5 * (lo[:-1] + lo[1:]), 0.5 * (la[:-1] + la[1:]))
    fields = {"hice": np.full(N, 0.3), "cice": np.full(N, 0.95), "u": np.zeros(N), "v": np.zeros(N),
              "uocean": np.zeros(N), "vocean": np.zeros(N), "ssh": np.zeros(N),
              "uwind": (12.0 * np.cos(4 * cy)).ravel(), "vwind": (6.0 * np.sin(3 * cx)).ravel()}
    out = {"mesh": f"{n}x{n} lon/lat cells, lon -0.3..0.3 rad, lat 1.0..1.3 rad"}
    for name, prec in (("fp64", 0), ("fp32", 1)):
        k = MEVPDynamicsKernel(dg_comp=DG, alpha=ALPHA, beta=BETA, n_steps=NSTEPS, precision=prec)
        k.initialise(coords, True, mask)
        for f, arr in fields.items():
            k.setData(f, arr)
        k.time_updates(DT, 3)
        steps = max(3, args.steps // 2)
        ms = k.time_updates(DT, steps) / steps
        kms, kname = k.time_kernel(0, 30)
        bpe = bytes_per_element_iteration_stress(4 if prec else 8, spherical=True)
        out[name] = {"value": N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "stress_kernel": kname,
                     "stress_kernel_ms": kms, "stress_GBps": N * bpe / (kms * 1e-3) / 1e9,
                     "algorithmic_bytes_per_element": bpe}
        k.close()
    return out


def ice_growth_variant(args, N: int):
    """The column thermodynamics step before the dynamics (IceGrowth with
    ThermoIce0, HiblerSpread, ConstantHealing) on the same number of cells:
    device time of repeated updates (the state evolves, forcing fixed), its
    algorithmic bytes against HBM, and the CPU oracle on the same inputs."""
    from nextsimdg_gb300.ice_growth import IceGrowth
    rng = np.random.default_rng(5)
    cice = rng.uniform(0.0, 1.0, N)
    fields = {"hice": rng.uniform(0.0, 3.0, N) * cice, "cice": cice, "hsnow": rng.uniform(0.0, 0.3, N) * cice,
              "tice": rng.uniform(-30.0, 0.0, N), "qia": rng.uniform(-100.0, 400.0, N),
              "dqia_dt": rng.uniform(0.0, 30.0, N), "qow": rng.uniform(-200.0, 400.0, N),
              "qio": rng.uniform(0.0, 200.0, N), "sublim": rng.uniform(-1e-5, 1e-5, N),
              "snowfall": rng.uniform(0.0, 1e-4, N), "penSW": rng.uniform(0.0, 50.0, N),
              "sst": rng.uniform(-1.8, 1.0, N), "tf": np.full(N, -1.751), "mlbhc": np.full(N, 4.29e7),
              "damage": rng.uniform(0.0, 1.0, N)}
    g = IceGrowth(N)
    for name, arr in fields.items():
        g.setData(name, arr)
    reps = 50
    g.time_updates(120.0, 5)
    ms = g.time_updates(120.0, reps) / reps
    g.close()
    bpe = 25 * 8 + 21 * 8 + 1  # slots read, slots written, ocean flag
    hbm, _ = measured_peaks()
    out = {"cells": N, "value": N / (ms * 1e-3), "unit": "cell-updates/s", "ms_per_update": ms,
           "algorithmic_bytes_per_cell": bpe, "achieved_GBps": N * bpe / (ms * 1e-3) / 1e9,
           "hbm_frac": N * bpe / (ms * 1e-3) / 1e9 / hbm, "parity": "bit-identical to the CPU oracle (tests)"}
    try:
        from oracle import pyoracle
        o = pyoracle.OracleIceGrowth(N)
        for name, arr in fields.items():
            o.setData(name, arr)
        t0 = time.perf_counter()
        n_cpu = 3
        for _ in range(n_cpu):
            o.update(120.0)
        cpu_s = (time.perf_counter() - t0) / n_cpu
        out["cpu_baseline"] = {"value": N / cpu_s, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                               "sample": f"{n_cpu} updates of {N} cells"}
    except Exception as ex:  # the oracle is test infrastructure: report, do not fail the bench
        out["cpu_baseline"] = {"unavailable": str(ex)[:200]}
    return out


def day_error(args, box, steps: int, alpha: float = ALPHA, every: int = 120, perturbed_runs: bool = False):
    """Velocity / thickness / concentration RMS against the FP64 path every
    `every` model steps up to `steps`: the headline precision path and the
    FP64 path with h scaled by (1 + 1e-14), the floor no implementation can
    go below.  mEVP with alpha = beta of a few hundred is far from converged on
    1 km cells (its iteration needs alpha beta well above zeta dt (pi / dx)^2
    / (rho h)), so a trajectory can go unstable; the library flags the
    non-finite velocity and the run is reported with the checkpoint at which
    it was flagged, not measured after it.  perturbed_runs adds the FP64 path
    with h x (1 + 2e-14) and the FP32 path with h x (1 + 1e-14): whether a
    run goes unstable within the day depends on the rounding that seeds the
    growing mode, in either precision."""
    from nextsimdg_gb300._lib import NsdgError
    from nextsimdg_gb300.boxtest import step_forcing
    ks = {"fp64": make_kernel(box, 0, alpha=alpha), "fp64_h_times_1p1e-14": make_kernel(box, 0, scale_h=1 + 1e-14,
                                                                                        alpha=alpha),
          "fp32": make_kernel(box, 1, alpha=alpha)}
    if perturbed_runs:
        ks["fp64_h_times_1p2e-14"] = make_kernel(box, 0, scale_h=1 + 2e-14, alpha=alpha)
        ks["fp32_h_times_1p1e-14"] = make_kernel(box, 1, scale_h=1 + 1e-14, alpha=alpha)
    compared = [n for n in ks if n != "fp64"]
    failed = {}
    rms = lambda a: float(np.sqrt(np.mean(a * a)))  # noqa: E731
    out = {"steps": steps, "simulated_hours": steps * DT / 3600.0, "alpha": alpha, "cells": box.nelements,
           "checkpoints": []}
    for s in range(steps):
        for n, k in ks.items():
            if n not in failed:
                step_forcing(k, box, s)
                k.update(s * DT, DT)
        if (s + 1) % every == 0 or s == steps - 1:
            r = {}
            for n, k in ks.items():
                if n in failed:
                    continue
                try:
                    r[n] = {f: k.getDG0Data(f) for f in ("u", "v", "hice", "cice")}
                except NsdgError:
                    failed[n] = s + 1
            cp = {"step": s + 1}
            for n in compared:
                if n in r and "fp64" in r:
                    x, ref = r[n], r["fp64"]
                    cp[n] = {"u_v_rms_m_per_s": rms(np.hypot(x["u"] - ref["u"], x["v"] - ref["v"])),
                             "h_rms_m": rms(x["hice"] - ref["hice"]), "A_rms": rms(x["cice"] - ref["cice"])}
            out["checkpoints"].append(cp)
    last = out["checkpoints"][-1]
    for n in compared:
        if n in last:
            out[n] = last[n]
        else:
            run = n if n in failed else "fp64"
            out[n] = {"non_finite_by_step": failed.get(run), "run": run}
    out["non_finite_by_step"] = dict(failed)
    for k in ks.values():
        k.close()
    return out


def e2e_cycle(k, box, args, world, pinned: bool = True, device_forcing: bool = False,
              batched: bool = False) -> dict:
    """The reference's module cycle through the C ABI with host buffers
    (MEVPDynamics::update, MEVPDynamics.cpp:59-87): setData of h, A, the
    winds, the ocean current and ssh, update, then getDG0Data of h, A, u, v
    and the ice-ocean stress; wall clock, host <-> device copies inside,
    median of three repetitions of the K steps.  pinned: page-locked host
    buffers (through torch) or the pageable numpy arrays a ModelArray-like
    caller holds.  device_forcing: the winds and the ocean current computed on
    the device (nsdg_kernel_benchmark_*), so each step copies only h, A and
    ssh in.  batched: the same step as one nsdg_kernel_module_step call (the
    same copies in and out, one wait; what the GPUMEVPDynamics module does)
    instead of 13 separate calls."""
    N = box.nelements
    if pinned:
        try:
            import torch
            pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        except Exception:
            pin = np.ascontiguousarray
    else:
        pin = lambda a: np.array(a, dtype=np.float64, copy=True)  # noqa: E731
    uo, vo = box.ocean()
    uo, vo, ssh = pin(uo), pin(vo), pin(box.ssh())
    start = args.warmup + args.steps
    winds = [tuple(pin(w) for w in box.wind(s * DT)) for s in range(start)] if not device_forcing else None
    h, a = pin(k.getDG0Data("hice")), pin(k.getDG0Data("cice"))
    outs = {n: pin(np.empty(N)) for n in ("hice", "cice", "u", "v", "uiostress", "viostress")}
    forcing = box.device_forcing() if device_forcing else None

    def cycle(s, kk=None):
        kk = k if kk is None else kk
        if batched and not device_forcing:
            kk.module_step(s * DT, DT, {"hice": outs["hice"] if s else h, "cice": outs["cice"] if s else a,
                                        "uwind": winds[s][0], "vwind": winds[s][1], "uocean": uo, "vocean": vo,
                                        "ssh": ssh}, outs)
            return
        kk.setData("hice", outs["hice"] if s else h)
        kk.setData("cice", outs["cice"] if s else a)
        if device_forcing:
            kk.benchmark_atmosphere(forcing, s * DT)
            if s == 0:
                kk.benchmark_ocean(forcing)
        else:
            kk.setData("uwind", winds[s][0])
            kk.setData("vwind", winds[s][1])
            kk.setData("uocean", uo)
            kk.setData("vocean", vo)
        kk.setData("ssh", ssh)
        kk.update(s * DT, DT)
        for n, buf in outs.items():
            kk.getDG0Data(n, out=buf)

    for s in range(args.warmup):
        cycle(s)
    # three timed repetitions of the K steps (the host shares its cores with
    # the rest of the box): the median is reported, every trial is kept
    trials = []
    for _ in range(3):
        dist_barrier(world)
        t0 = time.perf_counter()
        for s in range(args.warmup, args.warmup + args.steps):
            cycle(s)
        t_e2e = time.perf_counter() - t0
        dist_barrier(world)
        trials.append(dist_max(t_e2e, world))
    t = statistics.median(trials)
    copies_in = 3 if device_forcing else 7
    return {"value": world * N * args.steps / t, "unit": UNIT, "h2d_bytes_per_step": copies_in * N * 8,
            "d2h_bytes_per_step": 6 * N * 8, "trials": [world * N * args.steps / x for x in trials],
            "host_buffers": "pinned" if pinned else "pageable",
            "forcing": "device (nsdg_kernel_benchmark_*)" if device_forcing else "host, setData",
            "calls": "one nsdg_kernel_module_step per step" if batched and not device_forcing
            else "separate setData / update / getDG0Data calls",
            "timing": "median of 3 repetitions of the timed steps, wall clock", "cycle": cycle}


def run_ours(args, world, rank, local):
    from nextsimdg_gb300.boxtest import BoxTest

    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("CUDA_VISIBLE_DEVICES", str(local))
    prec = 1 if args.precision == "mixed" else 0
    box = BoxTest(args.nx)
    k = make_kernel(box, prec)
    N = box.nelements

    # ---- value: device-resident steps (CUDA graph replays, CUDA events) ----
    k.time_updates(DT, max(args.warmup, 3))
    dist_barrier(world)
    with ClockSampler(local) as clk:
        ms = k.time_updates(DT, args.steps)
    k.synchronize()
    dist_barrier(world)
    ms_max = dist_max(ms, world)
    value = world * N * args.steps / (ms_max * 1e-3)
    launches = k.launches_per_update()

    # ---- e2e: the module cycle through the C ABI, host buffers ----
    e2e_res = e2e_cycle(k, box, args, world, pinned=True)
    e2e_module_step = e2e_cycle(k, box, args, world, pinned=True, batched=True)
    e2e_pageable = e2e_cycle(k, box, args, world, pinned=False)
    # what the module adapters do with a model's (pageable) arrays: one
    # module-step call per step
    e2e_module_pageable = e2e_cycle(k, box, args, world, pinned=False, batched=True)
    e2e_device_forcing = e2e_cycle(k, box, args, world, pinned=True, device_forcing=True)
    e2e_calls = e2e_call_breakdown(k, e2e_res["cycle"], args.warmup, args.steps) if args.e2e_calls else None

    roof, node = stress_roofline(k, N, prec, ms_max / args.steps, local, args.nx)
    tiled = k.transport_variant()[0] == "tiled"
    launched = launched_bytes_per_cell_update(box, prec, (k.stress_variant()[0] or "fp64") if prec else "fp64",
                                              tiled_transport=tiled)
    transport = transport_record(k, N, ms_max / args.steps)
    k_host_direct = k.host_direct()
    k.close()

    variants = {}
    if not args.no_variants and world == 1:
        other = 0 if prec else 1
        ko = make_kernel(box, other)
        ko.time_updates(DT, 3)
        oms = ko.time_updates(DT, args.steps) / args.steps
        ko.synchronize()
        oroof, _ = stress_roofline(ko, N, other, oms, local, args.nx)
        oe2e = e2e_cycle(ko, box, args, world, pinned=True) if other == 0 else None
        oe2e_pageable = e2e_cycle(ko, box, args, world, pinned=False) if other == 0 else None
        ko.close()
        variants["plain_fp64" if prec else "mixed_fp32"] = {
            "value": N / (oms * 1e-3), "unit": UNIT, "ms_per_step": oms,
            "headline_speedup_over_this": oms / (ms_max / args.steps), "roofline": oroof,
            "launched_bytes_per_cell_update": launched_bytes_per_cell_update(box, other, "fp64"),
            **({"e2e": {kk: vv for kk, vv in oe2e.items() if kk != "cycle"},
                "e2e_pageable": {kk: vv for kk, vv in oe2e_pageable.items() if kk != "cycle"}} if oe2e else {})}
        if prec:
            variants["plain_fp64_pairs"] = fp64_pairs_variant(args, box, N, local)
            variants["distorted_mixed"] = distorted_variant(args, local)
            variants["ensemble32"] = ensemble_variant(args)
        if prec and args.warm_train_iters > 0:
            variants["learned_fp32"] = learned_config5_variant(args)
        if prec and not args.no_bbm:
            variants["bbm"] = bbm_variant(args, box, N)
        if prec:
            variants["spherical"] = spherical_variant(args, N, local)
            variants["ice_growth"] = ice_growth_variant(args, N)
    err = (day_error(args, box, args.error_steps, every=60, perturbed_runs=True)
           if (prec and args.error_steps > 0 and world == 1) else None)
    if err is not None and args.nx != 256:
        # the same day on 2 km cells with the reference's default relaxation,
        # where the plain mEVP stays stable
        from nextsimdg_gb300.boxtest import BoxTest as _Box
        err["box256_alpha1500"] = day_error(args, _Box(256), args.error_steps, alpha=1500.0)

    if rank == 0:
        base = cpu_baseline(args.nx) if world == 1 and not args.no_cpu_baseline else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == 0 else "f32+f64",
            "data": "synthetic box test",
            "config": {"workload": f"box test {args.nx}x{args.nx}, DG2 transport, CG2 velocity, mEVP {NSTEPS} "
                                   f"iterations, alpha=beta={ALPHA:g}, dt={DT:g} s",
                       "precision": args.precision,
                       "method": ("FP32 bulk (FP64: conservation sums, inverse mass matrices, Delta, viscosity); "
                                  "the learned warm start is measured in variants.learned_fp32 (1024 x 1024), not enabled here"
                                  if prec else "FP64 throughout (the reference's arithmetic)"),
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": ("inputs larger than L2, no flush: each step sweeps the FP64 DG state, RK stage "
                              "buffers, transport velocities and M^-1 diagonals (~125 MB at 512^2), besides the "
                              "sub-cycle's ~110 MB working set" if tiled else
                              "inputs larger than L2, no flush: each step sweeps the transport cell operators "
                              "(113 MB in FP32), the FP64 inverse mass matrices (75 MB) and the FP64 stage "
                              "buffers, besides the sub-cycle's ~110 MB working set"),
                       "bytes_per_cell_update_reference_layout": bytes_per_cell_update(word=4 if prec else 8),
                       "bytes_per_cell_update": launched["total"],
                       "bytes_per_cell_update_parts": launched,
                       "bytes_note": "bytes_per_cell_update counts the arrays the launched kernels move; "
                                     "the reference-layout figure (every per-element operator streamed, "
                                     "the unfused reference data flow) is the nominal upper figure"},
            "e2e": {**{kk: vv for kk, vv in e2e_res.items() if kk != "cycle"},
                    **({"calls_us": e2e_calls} if e2e_calls else {})},
            "e2e_module_step": {kk: vv for kk, vv in e2e_module_step.items() if kk != "cycle"},
            "e2e_pageable": {kk: vv for kk, vv in e2e_pageable.items() if kk != "cycle"},
            "e2e_module_step_pageable": {**{kk: vv for kk, vv in e2e_module_pageable.items() if kk != "cycle"},
                                         "host_direct": k_host_direct},
            "e2e_device_forcing": {kk: vv for kk, vv in e2e_device_forcing.items() if kk != "cycle"},
            "gpu_launches": launches * args.steps,
            "roofline": roof,
            "node_kernel": node,
            "transport_kernel": transport,
            "clocks": clk.summary(),
        }
        if err:
            line["velocity_error_vs_fp64"] = err
        if base:
            line["cpu_baseline"] = base
        if variants:
            line["variants"] = variants
        print(json.dumps(line), flush=True)


def e2e_call_breakdown(k, cycle, start: int, steps: int) -> dict:
    """Median wall-clock microseconds of each call of the module cycle
    (--e2e-calls): the calls of `cycle` are timed one by one, with an explicit
    wait for the step after `update` so that the first read times only its own
    work.  Runs after the timed region; not part of any reported rate."""
    samples: dict[str, list[float]] = {}

    class Timed:
        def __init__(self, inner):
            self._k = inner

        def __getattr__(self, name):
            fn = getattr(self._k, name)

            def timed(*a, **kw):
                label = f"{name}({a[0]})" if name in ("setData", "getDG0Data") else name
                t0 = time.perf_counter()
                r = fn(*a, **kw)
                if name == "update":
                    samples.setdefault("update (enqueue)", []).append((time.perf_counter() - t0) * 1e6)
                    t0 = time.perf_counter()
                    self._k.synchronize()
                    label = "wait for the step"
                samples.setdefault(label, []).append((time.perf_counter() - t0) * 1e6)
                return r
            return timed

    proxy = Timed(k)
    for s in range(start, start + steps):
        cycle(s, proxy)
    return {name: statistics.median(v) for name, v in samples.items()}


def ensemble_boxes(n_members: int, seed: int = 2024):
    """32-member ensemble of the box test: square sides drawn uniformly from
    {64, 128, 192, 256, 384}; cyclone start perturbed by up to +-50 km and
    speed 8-12 m/s; seeded Gaussian noise on h with sigma 0.02 m."""
    from nextsimdg_gb300.boxtest import BoxTest
    rng = np.random.default_rng(seed)
    sides = rng.choice([64, 128, 192, 256, 384], size=n_members)
    boxes = []
    for i, n in enumerate(sides):
        L = 512e3
        start = (0.5 * L + rng.uniform(-50e3, 50e3), 0.5 * L + rng.uniform(-50e3, 50e3))
        boxes.append(BoxTest(int(n), seed=int(seed + i), h_noise=0.02, start=start,
                             wind_speed=float(rng.uniform(8.0, 12.0))))
    return boxes


def ensemble_measure(args, n_members: int) -> dict:
    """Batched ensemble (one graph per step for all members) against the same
    members stepped one after another, each with its own graph."""
    from nextsimdg_gb300.dynamics import Ensemble, MEVPDynamicsKernel

    boxes = ensemble_boxes(n_members)
    members = []
    for b in boxes:
        k = MEVPDynamicsKernel(dg_comp=DG, alpha=ALPHA, beta=BETA, n_steps=NSTEPS, precision=1)
        k.initialise(b.coords(), False, b.mask())
        for name, arr in b.initial_fields().items():
            k.setData(name, arr)
        members.append(k)
    cells = sum(b.nelements for b in boxes)
    ens = Ensemble(members)
    ens.time_updates(DT, max(args.warmup, 3))
    with ClockSampler(0) as clk:
        ms = ens.time_updates(DT, args.steps)
    launches = ens.launches_per_update()
    # the sub-cycle as one persistent cooperative launch per step (every box
    # test is a parallelogram mesh)
    try:
        ens.set_persistent(True)
        ens.time_updates(DT, max(args.warmup, 3))
        pms = ens.time_updates(DT, args.steps)
        persistent = {"value": sum(b.nelements for b in boxes) * args.steps / (pms * 1e-3),
                      "ms_per_step": pms / args.steps, "gpu_launches_per_step": ens.launches_per_update()}
        ens.set_persistent(False)
    except Exception as exc:  # reported, not fatal for the other variants
        persistent = {"error": str(exc)}
    # the same members one by one (each its own graph, same stream order)
    t_seq = 0.0
    for k in members:
        k.time_updates(DT, 1)
        t_seq += k.time_updates(DT, args.steps)
    tiles = {}
    for i, b in enumerate(boxes):
        tiles[f"{b.nx}"] = "x".join(map(str, ens.tile(i)))
    out = {"value": cells * args.steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / args.steps, "cells": cells,
           "members": len(boxes), "sides": sorted(int(b.nx) for b in boxes),
           "sequential_members": {"value": cells * args.steps / (t_seq * 1e-3), "ms_per_step": t_seq / args.steps},
           "autotuned_tiles": tiles, "gpu_launches_per_step": launches, "persistent_subcycle": persistent,
           "clocks": clk.summary()}
    ens.close()
    for k in members:
        k.close()
    return out


def run_ensemble(args):
    r = ensemble_measure(args, args.ensemble)
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic box-test ensemble",
            "config": {"workload": f"ensemble of {r['members']} box tests, sides "
                                   f"{sorted(set(r['sides']))}, {r['cells']} cells, DG2, mEVP {NSTEPS} "
                                   f"iterations, mixed precision", "members": r["members"]},
            "sequential_members": r["sequential_members"], "autotuned_tiles": r["autotuned_tiles"],
            "gpu_launches": r["gpu_launches_per_step"] * args.steps, "clocks": r["clocks"]}
    print(json.dumps(line), flush=True)


def run_profile(args):
    """Setup plus warm-up and K device-resident steps, nothing else
    (--rheology bbm: the BBM box test with the elastic sub-steps the grid
    needs)."""
    from nextsimdg_gb300.boxtest import BoxTest
    from nextsimdg_gb300.dynamics import BBMDynamicsKernel, MEVPDynamicsKernel

    box = BoxTest(args.nx)
    prec = 1 if args.precision == "mixed" else 0
    if args.rheology == "bbm":
        dx = box.L / box.nx
        sub = max(NSTEPS, int(math.ceil(DT / (0.5 * dx / math.sqrt(5.9467e8 / 900.0)))))
        k = BBMDynamicsKernel(dg_comp=DG, n_steps=int(math.ceil(sub / 50.0)) * 50, precision=prec)
    else:
        k = MEVPDynamicsKernel(dg_comp=DG, alpha=ALPHA, beta=BETA, n_steps=NSTEPS, precision=prec)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    if args.rheology == "bbm":
        k.setData("damage", box.damage())
    for s in range(args.warmup + args.steps):
        k.update(s * DT, DT)
    k.synchronize()
    print(json.dumps({"profile": True, "steps": args.steps, "warmup": args.warmup,
                      "launches_per_step": k.launches_per_update()}))
    k.close()


def _oracle_rate(box, dg: int, rheology: int, n_steps: int, steps: int, threads: int | None = None,
                 warm: int = 1) -> dict:
    """The oracle stepping `box` (all OpenMP threads, or `threads`): cell-updates/s
    over `steps` model steps after `warm` untimed ones."""
    from oracle import pyoracle
    from nextsimdg_gb300.boxtest import step_forcing
    pyoracle.load()
    cores = pyoracle.num_threads()
    k = pyoracle.OracleKernel(rheology, dg, alpha=ALPHA, beta=BETA, n_steps=n_steps)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    if rheology == 1:
        k.setData("damage", box.damage())
    if threads:
        pyoracle.set_threads(threads)
    try:
        for s in range(warm):
            step_forcing(k, box, s)
            k.update(s * DT, DT)
        t = 0.0
        for s in range(warm, warm + steps):
            step_forcing(k, box, s)
            t0 = time.perf_counter()
            k.update(s * DT, DT)
            t += time.perf_counter() - t0
    finally:
        pyoracle.set_threads(cores)
    return {"value": box.nelements * steps / t, "steps": steps, "seconds": round(t, 2),
            "threads": threads or cores}


def _gpu_rate(box, dg: int, rheology: int, precision: int, n_steps: int, steps: int) -> dict:
    """The library's kernel stepping `box` as one CUDA graph per step (CUDA
    events, device-resident inputs)."""
    from nextsimdg_gb300.boxtest import step_forcing
    from nextsimdg_gb300.dynamics import BBMDynamicsKernel, MEVPDynamicsKernel
    if rheology == 1:
        k = BBMDynamicsKernel(dg_comp=dg, n_steps=n_steps, precision=precision)
    else:
        k = MEVPDynamicsKernel(dg_comp=dg, alpha=ALPHA, beta=BETA, n_steps=n_steps, precision=precision)
    k.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        k.setData(name, arr)
    if rheology == 1:
        k.setData("damage", box.damage())
    for s in range(3):
        step_forcing(k, box, s)
        k.update(s * DT, DT)
    ms = k.time_updates(DT, steps) / steps
    k.close()
    return {"value": box.nelements / (ms * 1e-3), "ms_per_step": ms, "steps": steps}


def run_table(args):
    """One JSON line per benchmark configuration: the oracle on the host cores
    (all threads and one thread) next to the GPU paths, same grid, same
    forcing.  The one-thread and large-grid CPU samples are bounded (a few
    steps); each entry states its sample."""
    from nextsimdg_gb300.boxtest import BoxTest
    from oracle import pyoracle
    pyoracle.load()
    host = {"cpu_model": cpu_model(), "cores": pyoracle.num_threads()}
    bbm_sub = lambda b: int(math.ceil(max(NSTEPS, math.ceil(  # noqa: E731
        DT / (0.5 * (b.L / b.nx) / math.sqrt(5.9467e8 / 900.0)))) / 50.0)) * 50
    rows = []
    b = BoxTest(64)
    rows.append({"config": "64x64 DG1/CG2 FP64, one day (720 steps)",
                 "cpu_all_cores": _oracle_rate(b, 1, 0, NSTEPS, 720),
                 "cpu_one_thread": _oracle_rate(b, 1, 0, NSTEPS, 20, threads=1),
                 "gpu_fp64": _gpu_rate(b, 1, 0, 0, NSTEPS, 720),
                 "gpu_mixed": _gpu_rate(b, 1, 0, 1, NSTEPS, 720)})
    b = BoxTest(256)
    rows.append({"config": "256x256 DG2/CG2 FP64",
                 "cpu_all_cores": _oracle_rate(b, DG, 0, NSTEPS, 10),
                 "cpu_one_thread": _oracle_rate(b, DG, 0, NSTEPS, 1, threads=1),
                 "gpu_fp64": _gpu_rate(b, DG, 0, 0, NSTEPS, 20),
                 "gpu_mixed": _gpu_rate(b, DG, 0, 1, NSTEPS, 20)})
    b = BoxTest(512)
    sub = bbm_sub(b)
    rows.append({"config": f"512x512 DG2/CG2: mEVP, and BBM with {sub} elastic sub-steps",
                 "cpu_all_cores": _oracle_rate(b, DG, 0, NSTEPS, 5),
                 "cpu_one_thread": _oracle_rate(b, DG, 0, NSTEPS, 1, threads=1, warm=0),
                 "cpu_all_cores_bbm": _oracle_rate(b, DG, 1, sub, 1),
                 "gpu_fp64": _gpu_rate(b, DG, 0, 0, NSTEPS, 10),
                 "gpu_mixed": _gpu_rate(b, DG, 0, 1, NSTEPS, 20),
                 "gpu_fp64_bbm": _gpu_rate(b, DG, 1, 0, sub, 3),
                 "gpu_mixed_bbm": _gpu_rate(b, DG, 1, 1, sub, 3)})
    boxes = ensemble_boxes(32)
    cells = sum(x.nelements for x in boxes)
    t_cpu = sum(x.nelements / _oracle_rate(x, DG, 0, NSTEPS, 1)["value"] for x in boxes)
    t_fp64 = sum(x.nelements / _gpu_rate(x, DG, 0, 0, NSTEPS, 3)["value"] for x in boxes)
    ens = ensemble_measure(args, 32)
    rows.append({"config": f"32-member uneven ensemble, {cells} cells",
                 "cpu_all_cores": {"value": cells / t_cpu, "steps": 1, "seconds": round(t_cpu, 2),
                                   "sample": "one step of every member after one warm-up step"},
                 "cpu_one_thread": None,
                 "gpu_fp64": {"value": cells / t_fp64, "sample": "members stepped one by one, FP64"},
                 "gpu_mixed": {kk: ens[kk] for kk in ("value", "ms_per_step", "persistent_subcycle")}})
    b = BoxTest(1024)
    rows.append({"config": "1024x1024 DG2/CG2 (the learned warm start's grid)",
                 "cpu_all_cores": _oracle_rate(b, DG, 0, NSTEPS, 1, warm=0),
                 "cpu_one_thread": None,
                 "gpu_fp64": _gpu_rate(b, DG, 0, 0, NSTEPS, 3),
                 "gpu_mixed": _gpu_rate(b, DG, 0, 1, NSTEPS, 10),
                 "gpu_learned": "variants.learned_fp32 of the default bench line"})
    for r in rows:
        print(json.dumps({"table": True, "unit": UNIT, **host, **r}), flush=True)


def run_net_forward(args):
    """The learned warm start's network (6 layers of 3x3 convolutions,
    64-48-48-48-48-48-32 channels, BF16 on the tensor cores, FP32
    accumulation) on one nx x nx grid: CUDA-event time per forward pass,
    its FLOPs (2 x 9 x c_in x c_out per cell and layer) and the fraction of
    the measured bf16 GEMM rate (burst: the pass is timed alone)."""
    from nextsimdg_gb300 import surrogate
    n = args.nx
    net = surrogate.warm_net(n, n, seed=1)
    x = np.random.default_rng(0).standard_normal((1, n, n, net.channels[0])).astype(np.float32)
    net.set_batch(x)
    net.time_forward(max(args.warmup, 3))
    ms = net.time_forward(args.steps)
    ch = net.channels
    flops = 2.0 * n * n * sum(9 * ch[i] * ch[i + 1] for i in range(len(ch) - 1))
    p = ROOT / "MEASURED_PEAKS.json"
    peak, kind = (json.loads(p.read_text()).get("bf16_tflops"), "measured") if p.exists() else (1900.0, "fallback")
    tf = flops / (ms * 1e-3) / 1e12
    print(json.dumps({"net_forward": True, "grid": f"{n}x{n}", "channels": list(ch), "ms_per_forward": ms,
                      "gflop_per_forward": flops / 1e9, "tflops": tf, "bf16_peak_tflops": peak,
                      "peak_kind": kind, "frac": tf / peak, "steps": args.steps}), flush=True)
    net.close()


def run_net_train(args):
    """One training step of the same network on one nx x nx grid (forward,
    loss, backward: the weight, bias and data gradients; the Adam update):
    wall-clock milliseconds per step (each step ends with the loss read back,
    so the steps do not overlap), after the warm-up steps."""
    from nextsimdg_gb300 import surrogate
    n = args.nx
    net = surrogate.warm_net(n, n, seed=1)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, n, n, net.channels[0])).astype(np.float32)
    t = rng.standard_normal((1, n, n, net.channels[-1])).astype(np.float32)
    net.set_batch(x, t, np.ones((1, n, n), dtype=np.float32))
    for _ in range(max(args.warmup, 3)):
        net.forward(copy=False)
        net.loss_backward()
        net.adam_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        net.forward(copy=False)
        net.loss_backward()
        net.adam_step()
    net.forward(copy=False)
    net.loss_backward()  # the last Adam update has been applied when this returns
    ms = (time.perf_counter() - t0) * 1e3 / (args.steps + 1)
    ch = net.channels
    flops = 3 * 2.0 * n * n * sum(9 * ch[i] * ch[i + 1] for i in range(len(ch) - 1))
    print(json.dumps({"net_train_step": True, "grid": f"{n}x{n}", "channels": list(ch), "ms_per_step": ms,
                      "gflop_per_step": flops / 1e9, "steps": args.steps,
                      "note": "forward + weight and data gradients (3 x the forward's GEMM FLOPs) + Adam"}),
          flush=True)
    net.close()


def _day_kernel(box, prec: int, env: dict | None = None, scale: float = 1.0, alpha: float = ALPHA):
    """make_kernel with the library's selection variables set while the
    kernel is created (they are read at creation)."""
    old = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})
    try:
        return make_kernel(box, prec, scale_h=scale, alpha=alpha)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def run_day_error(args):
    """Error checkpoints over a simulated day, one JSON line per checkpoint
    and a final RESULT line: RMS of u/v (as |(du, dv)|) and of the other
    fields against the plain FP64 path, for the FP64 path with h x (1 + 1e-14)
    (its own sensitivity, the floor) and the other paths.

    bbm:   512 x 512 BBM (damage 1, elastic sub-steps resolving the elastic
           wave), FP64 and mixed precision, 720 steps, every 120.
    parts: 256 x 256 mEVP alpha = beta = 1500: the mixed path, the mixed path
           with FP64 transport, the FP64 path with the float-pair stress
           kernel, 360 steps, every 60 (which part of the mixed path carries
           its excess over the floor).
    stability: 512 x 512 mEVP alpha = beta = 300 (the headline day), 720
           steps, every 60: the FP64 path with h x (1 + k 1e-14), k = 1..4,
           and the mixed path with each transport kernel and with h x
           (1 + k 1e-14), k = 1, 2: which of these runs the library flags as
           non-finite, and when (the configuration is near the mEVP's
           stability limit on 1 km cells)."""
    from nextsimdg_gb300._lib import NsdgError
    from nextsimdg_gb300.boxtest import BoxTest, step_forcing
    from nextsimdg_gb300.dynamics import BBMDynamicsKernel
    rms = lambda a: float(np.sqrt(np.mean(a * a)))  # noqa: E731
    if args.day_error == "stability":
        box = BoxTest(512)
        ks = {"fp64": _day_kernel(box, 0)}
        for j in range(1, 5):
            ks[f"fp64_h_x_1p{j}e-14"] = _day_kernel(box, 0, scale=1 + j * 1e-14)
        ks["mixed"] = _day_kernel(box, 1)
        ks["mixed_element_transport"] = _day_kernel(box, 1, {"NSDG_TRANSPORT_KERNEL": "element"})
        for j in (1, 2):
            ks[f"mixed_h_x_1p{j}e-14"] = _day_kernel(box, 1, scale=1 + j * 1e-14)
        steps, every, fields = 720, 60, ("u", "v", "hice", "cice")
        extra = {"grid": "512x512", "alpha": ALPHA}
    elif args.day_error == "parts":
        box = BoxTest(256)
        ks = {"fp64": _day_kernel(box, 0, alpha=1500.0), "fp64p": _day_kernel(box, 0, scale=1 + 1e-14, alpha=1500.0),
              "mixed": _day_kernel(box, 1, alpha=1500.0),
              "mixed_fp64_transport": _day_kernel(box, 1, {"NSDG_MIXED_TRANSPORT": "fp64"}, alpha=1500.0),
              "fp64_pairs": _day_kernel(box, 0, {"NSDG_FP64_STRESS": "pairs_tma"}, alpha=1500.0)}
        steps, every, fields = 360, 60, ("u", "v", "hice", "cice")
        extra = {"grid": "256x256", "alpha": 1500.0}
    else:
        box = BoxTest(512)
        dx = box.L / box.nx
        sub = max(NSTEPS, int(math.ceil(DT / (0.5 * dx / math.sqrt(5.9467e8 / 900.0)))))
        sub = int(math.ceil(sub / 50.0)) * 50
        ks = {}
        for name, prec, scale in (("fp64", 0, 1.0), ("fp64p", 0, 1.0 + 1e-14), ("mixed", 1, 1.0)):
            k = BBMDynamicsKernel(dg_comp=DG, n_steps=sub, precision=prec)
            k.initialise(box.coords(), False, box.mask())
            for f, arr in box.initial_fields().items():
                k.setData(f, arr * scale if f == "hice" else arr)
            k.setData("damage", box.damage())
            ks[name] = k
        steps, every, fields = 720, 120, ("u", "v", "hice", "cice", "damage")
        extra = {"grid": "512x512", "rheology": "BBM", "sub_steps": sub}
    failed, cps = {}, []
    t0 = time.time()
    for s in range(steps):
        for n, k in ks.items():
            if n not in failed:
                step_forcing(k, box, s)
                k.update(s * DT, DT)
        if (s + 1) % every == 0 or s == steps - 1:
            r = {}
            for n, k in ks.items():
                if n in failed:
                    continue
                try:
                    r[n] = {f: k.getDG0Data(f) for f in fields}
                except NsdgError:
                    failed[n] = s + 1
            cp = {"step": s + 1, "t": round(time.time() - t0, 1)}
            for n in ks:
                if n != "fp64" and n in r and "fp64" in r:
                    x, ref = r[n], r["fp64"]
                    cp[n] = {"uv": rms(np.hypot(x["u"] - ref["u"], x["v"] - ref["v"]))}
                    for f in fields:
                        if f not in ("u", "v"):
                            cp[n][f] = rms(x[f] - ref[f])
            cps.append(cp)
            print(json.dumps(cp), flush=True)
    for k in ks.values():
        k.close()
    print("RESULT", json.dumps({"day_error": args.day_error, **extra, "checkpoints": cps, "failed": failed}),
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--e2e-calls", action="store_true",
                    help="add e2e.calls_us: median microseconds of each call of the module cycle")
    ap.add_argument("--ensemble", type=int, default=0,
                    help="time a batched ensemble of this many box tests (mixed precision) instead")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="fp64: every operation FP64 (the reference's arithmetic); mixed: FP32 bulk")
    ap.add_argument("--nx", type=int, default=NX, help="box side in cells (512: the mixed-precision benchmark grid)")
    ap.add_argument("--error-steps", type=int, default=720,
                    help="model steps of the FP32-vs-FP64 velocity error check (720 = one day; 0: skip)")
    ap.add_argument("--warm-iters", type=int, default=40, help="mEVP iterations after the learned warm start")
    ap.add_argument("--warm-samples", type=int, default=120, help="training samples (every 3rd step)")
    ap.add_argument("--warm-train-iters", type=int, default=2000, help="Adam steps (0: skip the learned variant)")
    ap.add_argument("--no-bbm", action="store_true", help="skip the BBM variant")
    ap.add_argument("--day-error", choices=["bbm", "parts", "stability"],
                    help="error checkpoints over a simulated day against the FP64 path (BBM at 512^2, the "
                         "mixed path's parts at 256^2, or perturbed FP64 and mixed runs of the 512^2 day)")
    ap.add_argument("--net-train", action="store_true",
                    help="time one training step of the learned warm start's network on the --nx grid instead")
    ap.add_argument("--net-forward", action="store_true",
                    help="time the learned warm start's network forward pass on the --nx grid instead")
    ap.add_argument("--table", action="store_true",
                    help="one line per benchmark configuration: the oracle (all threads, one thread) beside the GPU")
    ap.add_argument("--profile", action="store_true",
                    help="only the device-resident steps (for ncu captures): no e2e, no baselines")
    ap.add_argument("--rheology", default="mevp", choices=["mevp", "bbm"], help="the rheology of --profile")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world, rank, local = dist_setup()
    if args.net_forward:
        run_net_forward(args)
    elif args.net_train:
        run_net_train(args)
    elif args.day_error:
        run_day_error(args)
    elif args.table:
        run_table(args)
    elif args.ensemble:
        run_ensemble(args)
    elif args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
