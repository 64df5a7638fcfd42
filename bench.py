"""Benchmark: DOF-stage updates/s of the DG tendency + LSRK54 hot path.

Workload: the dry rising thermal bubble on a 2500 m cube, 20x20x20 elements,
N=4 (1,000,000 nodes, 5,000,000 DOF), periodic in x and y, FreeSlip /
Insulating walls at the bottom and top, FlatOrientation + Gravity,
HydrostaticState(DryAdiabatic, theta0 = 300 K), +2 K cos^2 bubble of radius
250 m centred 350 m above the bottom, dt from CFL 0.4.  A step is one
LSRK54 step (5 fused tendency + stage kernels over the whole mesh).

value      mixed FP32/FP64 path (FP32 perturbation state, FP64 RK register),
           whole-job DOF-stage/s over all ranks, state resident in HBM; L2 is
           flushed (256 MiB write) between timed steps and each step is timed
           with CUDA events on the launching stream.  After W warm-up steps a
           leg times R regions of exactly K steps, each restarting from the
           initial state outside the region, R chosen so that the regions
           cover about a second (the clock samples then see the load); the
           median region gives ms_per_step.
fp64       the plain FP64 path, measured the same way.
e2e        the same metric through the C ABI with the FP64 state in pinned
           host memory (cmdg_lsrk54_step_mixed_host): each step reads the
           state from host memory over the host link (NVLink-C2C on GB300)
           into the device's FP32 perturbation, runs the step and writes the
           FP64 result back into host memory, all inside the timed region.
roofline   the dominant kernel (the fused mixed stage kernel) against the
           measured HBM copy bandwidth; algorithmic bytes per node-stage
           B = 2*5*4 (state r/w, FP32) + 2*5*8 (RK register r/w, FP64) = 120.
cpu_baseline  the C++ oracle (the CPU restatement of the reference) on the
           host cores, on a bounded sample of the same workload.
accuracy   outside the timed region: the mixed and FP64 GPU paths against the
           FP64 oracle after one tendency and after 100 LSRK54 steps (relative
           L2 and max relative error per field), and the mass and energy drift.
ensemble   the batched mixed ensemble of --workload ensemble (64 members),
           timed over the same steps (--no-ensemble skips it).

--impl reference times the reference's CPU path (the oracle port, the
reference itself is Julia and cannot run here) on the same workload.

--workload selects another configuration for the same measurement (the
default, the line the benchmark contract reads, is the bubble above):
  bubble-arrays  the bubble above through the reference's own grid arrays
            (vgeo, vmap+, elemtobndy in BrickTopology's Hilbert element order,
            cmdg_mesh_create_arrays): the path a Julia caller drops in;
            algorithmic bytes 202.4 (mixed) / 300.8 (FP64) per node-stage
            (the per-node geometry and reference words, the facing-node and
            reference-jump tables on top of the state and register)
  gcm       cubed-shell GCM, 6 x 12 x 12 x 6 elements, N=4 (648,000 nodes),
            30 km lid, isothermal 285 K, seeded zonal wind + 1 K anomaly;
            algorithmic bytes 224 (mixed) / 264 (FP64) per node-stage
  les       SmagorinskyLilly LES, 32 x 32 x 16 elements, N=4 (2,048,000
            nodes), N_bv = 0.01 1/s, seeded k^-5/3 velocity; 200 / 320 B
  hyper     the bubble above with DryBiharmonic hyperdiffusion (tau = 1 h):
            per stage the gradient, laplacian and gradient-of-laplacian passes
            and the stage kernel with hyperdiffusive fluxes; 308 / 536 B
  les16     16 members of the LES above (32.8 M nodes), mixed, batched
            (one graph per call) vs 16 sequential single-member solves
  ensemble  64 seeded rising-bubble members of 8^3..16^3 elements and
            N = 3..5, mixed; batched (one graph of per-order launches) vs
            64 sequential single-member solves
  hevi      the acoustic wave on the sphere of acousticwave_1d_imex.jl
            (N = 5, 10 x 10 x 6 x 5 cubed-shell elements, 648,000 nodes,
            FP64): ARK2GiraldoKellyConstantinescu steps of 100 s with the
            vertical acoustic-gravity linear model solved by the column LU;
            a stage is one of the 3 explicit stages of a step; the roofline
            kernel is the band substitution, algorithmic bytes = the
            structurally non-zero factor entries + the state words it moves

Multi-GPU: replicas only — each rank advances its own bubble; value is the
sum over ranks of the work divided by the slowest rank's time.
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

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "climatemachine.jl_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

NE = (20, 20, 20)
N = 4
L = 2500.0
CFL = 0.4
NSTAGE = 5
NFIELD = 5
BYTES_MIXED = 2 * 5 * 4 + 2 * 5 * 8   # per node-stage
BYTES_FP64 = 2 * 5 * 8 + 2 * 5 * 8
MIN_TIMED_S = 1.0    # each timed leg repeats its K-step region to cover about this much time
MAX_REPEATS = 400
WORKLOAD = ("rising bubble: 20x20x20 elements, N=4 (1e6 nodes, 5e6 DOF), [0,2500 m]^3, periodic x/y, "
            "FreeSlip walls z, dry Euler + gravity, HydrostaticState(DryAdiabatic 300 K), +2 K cos^2 bubble "
            "r=250 m at z=350 m, Rusanov, LSRK54 at CFL 0.4")


WORKLOADS = {
    "bubble": dict(desc=WORKLOAD, bytes_mixed=BYTES_MIXED, bytes_fp64=BYTES_FP64, launches_per_stage=1,
                   kernel="stage_kernel<4,float,mixed,stage>", profile="stage_kernel_mixed_bubble20.md"),
    "gcm": dict(desc="cubed-shell GCM: 6x12x12x6 elements, N=4 (648,000 nodes), R=6.371e6 m, 30 km lid, walls, "
                     "SphericalOrientation + gravity, HydrostaticState(Isothermal 285 K), seeded zonal wind 0-30 m/s "
                     "+ 1 K Gaussian anomaly, Rusanov, LSRK54 at CFL 0.4",
                bytes_mixed=224, bytes_fp64=264, launches_per_stage=1,
                kernel="shell_stage_kernel<4,float,mixed,stage>", profile="shell_stage_kernel_mixed_gcm.md"),
    "les": dict(desc="SmagorinskyLilly LES: 32x32x16 elements, N=4 (2,048,000 nodes), 3200x3200x1600 m, periodic "
                     "x/y, walls z, N_bv=0.01 1/s, seeded k^-5/3 velocity rms 1 m/s, Rusanov, LSRK54 at CFL 0.4",
                bytes_mixed=200, bytes_fp64=320, launches_per_stage=2,
                kernel="gradient_kernel + viscous_stage_kernel<4,float,mixed,stage,smagorinsky>",
                profile="viscous_stage_kernel_mixed_les.md"),
    # per node-stage: state + register 120 (mixed) / 160 (FP64), the per-node geometry and reference
    # words 17 x 4 / 17 x 8, the facing-node table 1.2 x 4 and (mixed, Rusanov) the reference-jump
    # table 1.2 x 8
    "bubble-arrays": dict(desc=WORKLOAD + "; grid arrays (vgeo, vmap+, elemtobndy) in BrickTopology's Hilbert "
                                          "element order through cmdg_mesh_create_arrays",
                          bytes_mixed=120 + 68 + 4.8 + 9.6, bytes_fp64=160 + 136 + 4.8, launches_per_stage=1,
                          kernel="arrays_stage_kernel<4,float,mixed,stage>",
                          profile="arrays_stage_kernel_mixed_bubble20.md"),
    # per node-stage: stage kernel 120 + nu grad^3 read 36; gradient pass 20 + 36; laplacian 36 + 12;
    # gradient of the laplacian 12 + 36 (FP32 words; FP64 doubles all but the RK register's 80)
    "hyper": dict(desc="rising bubble of the default workload with DryBiharmonic(tau = 3600 s) hyperdiffusion: "
                       "20x20x20 elements, N=4 (1e6 nodes), Rusanov, LSRK54 at CFL 0.4",
                  bytes_mixed=308, bytes_fp64=536, launches_per_stage=4,
                  kernel="hyperdiffusion passes + viscous_stage_kernel<4,float,mixed,stage,none,hyper>",
                  profile="hyper_passes_mixed_bubble20.md"),
}


def measure_ensemble(args, cmdg, workloads, torch, barrier, stream, flush):
    """64 seeded bubble members (8^3..16^3 elements, N = 3..5), mixed:
    batched steps (one CUDA graph per call, the tiling the autotuner picks)
    against 64 sequential single-member solves (each member autotuned, one
    graph-captured call per member).  Returns the ensemble's JSON fields."""
    specs = workloads.bubble_ensemble_specs(n=64)
    pairs = [workloads.bubble_member(s) for s in specs]
    dgs = [p[0] for p in pairs]
    Q0s = [dg.init_ode_state(Q0) for dg, Q0 in pairs]
    dts = [dg.courant_dt(dg.from_perturbation(Q), CFL) for dg, Q in zip(dgs, Q0s)]
    nodes = sum(dg.grid.nelem * dg.grid.Np for dg in dgs)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        barrier()
        ms = []
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            ms.append((a, b))
        barrier()
        return sum(a.elapsed_time(b) for a, b in ms)

    Qs = [Q.clone() for Q in Q0s]
    lsrks = [cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt) for dg, Q, dt in zip(dgs, Qs, dts)]
    for dg in dgs:
        dg.autotune(reps=3)

    def seq():
        for Q, lsrk in zip(Qs, lsrks):
            cmdg.dostep_(Q, lsrk, None, 0.0)

    ens = cmdg.Ensemble(dgs)
    Qe = [Q.clone() for Q in Q0s]
    dQe = [torch.zeros(Q.shape, dtype=torch.float64, device="cuda") for Q in Qe]
    cand_ms, tiling = ens.autotune(Qe, dQe, reps=5)
    persistent = tiling["kernel"][0] == "persistent"

    def bat():
        ens.lsrk54_step(Qe, dQe, dts, nsteps=1)

    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms_b = timed(bat)
    ms_s = timed(seq)
    work = NFIELD * nodes * NSTAGE * args.steps
    peak, peak_kind = measured_peak()
    ach = BYTES_MIXED * nodes / (ms_b / args.steps / NSTAGE * 1e-3) / 1e9
    return {"value": work / (ms_b * 1e-3), "unit": "DOF-stage/s", "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_b / args.steps,
            "workload": "64-member rising-bubble ensemble, elements U{8..16}^3, N U{3,4,5}, amplitude "
                        "U[0.5,3] K, radius U[150,400] m, mixed",
            "nodes": nodes, "tiling": {str(k): v for k, v in tiling.items()},
            "sequential": {"value": work / (ms_s * 1e-3), "ms_per_step": ms_s / args.steps},
            "speedup_vs_sequential": ms_s / ms_b,
            "autotune_ms_per_stage": {"per_order_family": cand_ms["per_order"],
                                      "persistent_best": min(cand_ms["persistent"])},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "peak_source": peak_kind,
                         "kernel": ("ens_lines_kernel (one persistent launch per stage, every order)"
                                    if persistent else "batch_stage_kernel<N> (one launch per order and stage)"),
                         "bytes_per_node_stage": BYTES_MIXED},
            "gpu_launches": args.steps * NSTAGE * (1 if persistent else 3), "clocks": clk.summary()}


def bench_ensemble(args, cmdg, workloads, torch, barrier, stream, flush):
    """The ensemble of measure_ensemble as its own JSON line."""
    r = measure_ensemble(args, cmdg, workloads, torch, barrier, stream, flush)
    line = {"metric": "DOF-stage updates/s", "value": r["value"], "unit": "DOF-stage/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": r["workload"], "nodes": r["nodes"], "tiling": r["tiling"],
                       "l2": "256 MiB buffer written between timed steps"}}
    for k in ("sequential", "speedup_vs_sequential", "autotune_ms_per_stage", "roofline", "gpu_launches", "clocks"):
        line[k] = r[k]
    print(json.dumps(line))
    return 0


def bench_les16(args, cmdg, workloads, torch, barrier, stream, flush):
    """The 16-member LES configuration: 16 SmagorinskyLilly members of
    32 x 32 x 16 elements, N = 4 (2,048,000 nodes each, 32.8 M in total),
    seeded k^-5/3 velocity fields (one seed per member) over an N_bv = 0.01
    stratification, mixed FP32/FP64, batched (one CUDA graph per call, the
    gradient pass and the viscous stage kernel of every member and stage)
    against 16 sequential single-member solves."""
    nmem = 16
    dgs = [workloads.les_model(precision="mixed") for _ in range(nmem)]
    xyz = dgs[0].grid.coordinates()
    Q0s = [workloads.les_initial_state(xyz, seed=2024 + m) for m in range(nmem)]
    Qs = [dg.init_ode_state(Q0) for dg, Q0 in zip(dgs, Q0s)]
    dt = min(dg.courant_dt(Q, CFL) for dg, Q in zip(dgs, Qs))
    nodes = sum(dg.grid.nelem * dg.grid.Np for dg in dgs)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        barrier()
        ms = []
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            ms.append((a, b))
        barrier()
        return sum(a.elapsed_time(b) for a, b in ms)

    ens = cmdg.Ensemble(dgs)
    dQe = [torch.zeros(Q.shape, dtype=torch.float64, device="cuda") for Q in Qs]
    Qseq = [Q.clone() for Q in Qs]
    lsrks = [cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt) for dg, Q in zip(dgs, Qseq)]

    def bat():
        ens.lsrk54_step(Qs, dQe, [dt] * nmem, nsteps=1)

    def seq():
        for Q, lsrk in zip(Qseq, lsrks):
            cmdg.dostep_(Q, lsrk, None, 0.0)

    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms_b = timed(bat)
    ms_s = timed(seq)
    # both runs took the same steps from the same states: the same numbers
    same = all(bool(torch.equal(a, b)) for a, b in zip(Qs, Qseq))
    work = NFIELD * nodes * NSTAGE * args.steps
    peak, peak_kind = measured_peak()
    bytes_ns = WORKLOADS["les"]["bytes_mixed"]
    ach = bytes_ns * nodes / (ms_b / args.steps / NSTAGE * 1e-3) / 1e9
    line = {"metric": "DOF-stage updates/s", "value": work / (ms_b * 1e-3), "unit": "DOF-stage/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_b / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "16-member SmagorinskyLilly LES ensemble: 32x32x16 elements, N=4 per member "
                                   "(2,048,000 nodes each), N_bv=0.01 1/s, seeded k^-5/3 velocity rms 1 m/s, mixed",
                       "l2": L2_NOTE, "parallelism": "replicas x1"},
            "nodes": nodes, "dt": dt,
            "sequential": {"value": work / (ms_s * 1e-3), "ms_per_step": ms_s / args.steps},
            "speedup_vs_sequential": ms_s / ms_b, "batched_equals_sequential": same,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "peak_source": peak_kind, "kernel": "gradient_kernel + viscous_stage_kernel (16 members)",
                         "bytes_per_node_stage": bytes_ns},
            "gpu_launches": args.steps * NSTAGE * 2 * nmem, "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def bench_hevi(args, cmdg, workloads, torch, barrier, stream, flush):
    """ARK2 + column-LU (HEVI) steps of the acoustic wave on the sphere: the
    explicit tendency of a mixed model (value: the fused remainder f - l of
    the vertical linear model on the FP32 perturbation plus the FP64 linear
    tendency) and in FP64 (fp64), the stage algebra and the column solve FP64
    in both;
    beside it the explicit LSRK54 path of the same mixed model at its own
    Courant time step, as simulated seconds per wall-clock second."""
    import numpy as np

    dt, _ = workloads.acoustic_wave_dt()

    def setup(precision):
        dg = workloads.acoustic_wave_model(precision=precision)
        Q0 = workloads.acoustic_wave_state(dg.grid.coordinates(), dg.reference_state()[:, 2])
        lin = cmdg.DGModel(cmdg.AtmosAcousticGravityLinearModel(dg.balance_law), dg.grid, direction="vertical",
                           state_auxiliary=dg)
        Q = torch.from_numpy(Q0).to("cuda")
        ark = cmdg.ARK2GiraldoKellyConstantinescu(dg, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                                  dt=dt)
        return dg, Q0, lin, Q, ark

    # a step is the reference test's step: one ARK2 step followed by the
    # vertical ExponentialFilter(grid, 0, 18) of every field (its callback);
    # the FP64 state is filtered by an FP64 model in both runs
    from cmdg.filters import ExponentialFilter, apply_

    def timed_steps(Q, ark, dgf, filt):
        def step():
            cmdg.dostep_(Q, ark, None, 0.0, 1)
            apply_(Q, (0, 1, 2, 3, 4), dgf, filt, direction="vertical")

        for _ in range(args.warmup):
            step()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        barrier()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        barrier()
        return sum(a.elapsed_time(b) for a, b in ev)

    dg, Q0, lin, Q, ark = setup("mixed")
    dg64, _, _, Q64, ark64 = setup("fp64")
    nodes = dg.grid.nelem * dg.grid.Np
    nz = dg.grid.ne[2]
    NB = 5 * (dg.grid.N + 1)
    fwd = sum(NB - 1 - max(0, p - 5) for p in range(NB))
    bwd = sum((NB - 1 if p < 5 else p) + 1 for p in range(NB))
    solve_bytes = 8 * ark.nline * (fwd + bwd) * nz + 8 * 5 * nodes * 5  # factors + b, y (w, r), out (r, w)

    filt = ExponentialFilter(dg64.grid, 0, 18)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = timed_steps(Q, ark, dg64, filt)
        ms64 = timed_steps(Q64, ark64, dg64, filt)
    M = dg64.grid.mass()
    a, b = Q.cpu().numpy(), Q64.cpu().numpy()
    rel = [math.sqrt(float(np.sum((a[:, sl] - b[:, sl]) ** 2 * M[:, None, :]))) /
           math.sqrt(float(np.sum(b[:, sl] ** 2 * M[:, None, :]))) for sl in (slice(0, 1), slice(1, 4), slice(4, 5))]
    # the substitution alone (2 of the launches of a step)
    X = dg.new_state(torch.float64)
    Qh = Q.clone()
    for _ in range(3):
        ark.backward_euler_solve(X, Qh)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    s0.record(stream)
    for _ in range(20):
        ark.backward_euler_solve(X, Qh)
    s1.record(stream)
    barrier()
    solve_ms = s0.elapsed_time(s1) / 20
    # e2e: the FP64 state in pinned host memory, copied in and out every step
    host = torch.from_numpy(np.ascontiguousarray(Q0)).pin_memory()
    Qd = torch.from_numpy(Q0).to("cuda")

    def e2e_step():
        Qd.copy_(host, non_blocking=True)
        cmdg.dostep_(Qd, ark, None, 0.0, 1)
        apply_(Qd, (0, 1, 2, 3, 4), dg64, filt, direction="vertical")
        host.copy_(Qd, non_blocking=True)

    for _ in range(2):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    ms_e2e = e0.elapsed_time(e1)
    # the explicit alternative: LSRK54 of the mixed model at its Courant time step
    Qx = dg.to_perturbation(torch.from_numpy(Q0).to("cuda"))
    dt_x = dg.courant_dt(Qx, CFL)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qx, dt=dt_x)
    nx = 50
    cmdg.dostep_(Qx, lsrk, None, 0.0, 3)
    x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    x0.record(stream)
    cmdg.dostep_(Qx, lsrk, None, 0.0, nx)
    x1.record(stream)
    barrier()
    ms_x = x0.elapsed_time(x1)

    cpu = None
    if not args.no_cpu_baseline:
        try:
            sys.path.insert(0, os.path.join(REPO, "oracle"))
            import oracle as O

            O.set_threads(os.cpu_count())
            R = O.EARTH["planet_radius"]
            om = O.OracleModel(5, shell=dict(nhorz=10, nvert=5, r_inner=R, r_outer=R + 10e3), orientation="sphere",
                               gravity=True, ref_state=True, profile="isothermal", T_surface=300.0)
            ohv = O.OracleHevi(om, dt)
            Qo = np.ascontiguousarray(Q0)
            t0 = time.perf_counter()
            ohv.step(Qo, 2)
            el = time.perf_counter() - t0
            cpu = {"value": NFIELD * om.nelem * om.Np * 3 * 2 / el, "unit": "DOF-stage/s", "cores": os.cpu_count(),
                   "kind": "port", "sample": "2 ARK2 steps of the full acoustic-wave mesh, FP64 oracle "
                                             "(factorization excluded)"}
        except Exception as exc:
            cpu = {"value": None, "error": str(exc)[:200]}

    work = NFIELD * nodes * 3 * args.steps
    peak, peak_kind = measured_peak()
    ach = solve_bytes / (solve_ms * 1e-3) / 1e9
    traffic = profile_traffic("hevi_band_solve_acoustic_wave.md")
    line = {"metric": "DOF-stage updates/s", "value": work / (ms * 1e-3), "unit": "DOF-stage/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "acoustic wave on the sphere (acousticwave_1d_imex.jl): cubed shell 6x10x10x5, "
                                   "N=5 (648,000 nodes), 10 km lid, isothermal 300 K, HEVI "
                                   "ARK2GiraldoKellyConstantinescu, dt = 100 s, ManyColumnLU",
                       "path": "explicit tendency: the fused remainder f - l on the FP32 perturbation plus the "
                               "FP64 linear tendency of the FP64 perturbation; ARK algebra, linear operator and "
                               "column LU FP64",
                       "dt": dt, "stages_per_step": 3, "column_lines": ark.nline, "band_half_width": ark.bandwidth,
                       "l2": "256 MiB buffer written between timed steps"},
            "fp64": {"value": work / (ms64 * 1e-3), "ms_per_step": ms64 / args.steps},
            "mixed_vs_fp64_rel_l2_rho_rhou_rhoe": rel,
            "mixed_vs_fp64_steps": args.warmup + args.steps,
            "step": "ARK2 step + vertical ExponentialFilter(grid, 0, 18) of every field (acousticwave_1d_imex.jl)",
            "simulated_s_per_wall_s": dt * args.steps / (ms * 1e-3),
            "explicit_lsrk54_mixed": {"dt": dt_x, "ms_per_step": ms_x / nx,
                                      "simulated_s_per_wall_s": dt_x * nx / (ms_x * 1e-3)},
            "column_solve_ms": solve_ms,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": traffic, "peak_source": peak_kind, "kernel": "band_solve_kernel<6>",
                         "bytes_per_solve": solve_bytes},
            "cpu_baseline": cpu,
            "e2e": {"value": work / (ms_e2e * 1e-3), "unit": "DOF-stage/s", "h2d_bytes_per_step": int(host.numel() * 8),
                    "d2h_bytes_per_step": int(host.numel() * 8)},
            "gpu_launches": args.steps * 13, "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def profile_traffic(name):
    """DRAM bytes per launch of a profiled kernel, from its summary under profiles/."""
    path = os.path.join(REPO, "profiles", name)
    if os.path.exists(path):
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


def profile_value(name, key):
    """A `key: value` figure of a profile summary under profiles/ (None when absent)."""
    path = os.path.join(REPO, "profiles", name)
    if os.path.exists(path):
        for line in open(path):
            if line.startswith(key + ":"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.proc = None
        self.index = index
        self.path = os.path.join(tempfile.gettempdir(), f"cmdg_clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return None
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 7:
                    try:
                        rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
                    except ValueError:
                        pass
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def cpu_reference_case(O, workload):
    """The oracle's model and FP64 initial state of a bench workload (the
    same configuration and seeded state as the GPU legs)."""
    import numpy as np

    bubble = dict(periodic=(1, 1, 0), orientation="flat", gravity=True, ref_state=True, profile="dry_adiabatic",
                  T_surface=300.0, T_min=0.0)
    if workload in ("bubble", "bubble-arrays", "hyper"):
        extra = dict(hyperdiffusion="dry_biharmonic", tau_hyper=3600.0) if workload == "hyper" else {}
        om = O.OracleModel(N, NE, (0, 0, 0), (L, L, L), **bubble, **extra)
        return om, om.init_bubble(theta0=300.0, amp=2.0, rc=250.0, xc=1250.0, yc=1250.0, zc=350.0)
    from cmdg import workloads

    if workload == "gcm":
        R = O.EARTH["planet_radius"]
        om = O.OracleModel(N, shell=dict(nhorz=12, nvert=6, r_inner=R, r_outer=R + 30e3), orientation="sphere",
                           gravity=True, ref_state=True, profile="isothermal", T_surface=285.0)
        return om, workloads.gcm_initial_state(np.ascontiguousarray(om.aux[:, 0:3]))
    if workload == "les":
        om = O.OracleModel(N, (32, 32, 16), (0, 0, 0), (3200.0, 3200.0, 1600.0), **bubble, turbulence="smagorinsky")
        return om, workloads.les_initial_state(np.ascontiguousarray(om.aux[:, 0:3]))
    raise ValueError(f"no CPU reference case for workload {workload!r}")


def run_cpu_reference(steps, threads=None, sample_steps=None, warmup=1, max_sec=None, workload="bubble"):
    """Times the oracle (CPU restatement of the reference) on the workload."""
    import numpy as np

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    threads = threads or os.cpu_count()
    O.set_threads(threads)
    om, Q = cpu_reference_case(O, workload)
    Q = np.ascontiguousarray(Q)
    dt = om.courant_dt(Q, CFL)
    dQ = om.state()
    w0 = time.perf_counter()
    om.lsrk54(Q, dt, max(1, warmup), dQ=dQ)  # warm-up
    per_step = (time.perf_counter() - w0) / max(1, warmup)
    nsteps = sample_steps or steps
    if max_sec is not None:
        # bounded: as many of the requested steps as fit in max_sec
        nsteps = max(1, min(nsteps, int(max_sec / max(per_step, 1e-9))))
    t0 = time.perf_counter()
    om.lsrk54(Q, dt, nsteps, dQ=dQ)
    el = time.perf_counter() - t0
    nodes = om.nelem * om.Np
    return dict(value=NFIELD * nodes * NSTAGE * nsteps / el, sec=el, steps=nsteps, threads=threads,
                warmup=max(1, warmup))


ACCURACY_STEPS = 100
L2_NOTE = ("GPU arm: a 256 MiB buffer is written between timed steps (L2 is 129 MB); CPU arm: the FP64 state and "
           "its working arrays (hundreds of MB) exceed the host caches")


def field_errors(got, ref, M, base=None):
    """Per-field errors of a state (nelem, 5, Np) against a reference state:
    relative L2 weighted by the mass matrix (euclidean_distance / norm,
    src/Arrays/MPIStateArrays.jl:583-648), max relative (max |got - ref| /
    max |ref|), and, with a base state, the L2 error relative to the change
    of the reference from that base (how well the evolution itself is
    reproduced)."""
    import numpy as np

    out = {"rel_l2": [], "max_rel": []}
    if base is not None:
        out["rel_l2_of_change"] = []
    for s in range(NFIELD):
        d = got[:, s] - ref[:, s]
        num = math.sqrt(float(np.sum(d * d * M)))
        den = math.sqrt(float(np.sum(ref[:, s] * ref[:, s] * M)))
        out["rel_l2"].append(num / den if den > 0 else num)
        mx = float(np.abs(ref[:, s]).max())
        out["max_rel"].append(float(np.abs(d).max()) / mx if mx > 0 else float(np.abs(d).max()))
        if base is not None:
            c = ref[:, s] - base[:, s]
            dc = math.sqrt(float(np.sum(c * c * M)))
            out["rel_l2_of_change"].append(num / dc if dc > 0 else None)
    # field groups rho, momentum as one vector, rho e (a momentum component
    # that is nearly zero, the vertical wind of a balanced state, carries the
    # others' rounding relative to its own tiny norm)
    out["rel_l2_rho_rhou_rhoe"] = []
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
        d = got[:, sl] - ref[:, sl]
        num = math.sqrt(float(np.sum(d * d * M[:, None, :])))
        den = math.sqrt(float(np.sum(ref[:, sl] * ref[:, sl] * M[:, None, :])))
        out["rel_l2_rho_rhou_rhoe"].append(num / den if den > 0 else num)
    return out


def accuracy_report(cmdg, torch, dg64, dgmx, Q0, dt, workload="bubble", steps=ACCURACY_STEPS):
    """Both GPU paths against the FP64 oracle (the CPU restatement of the
    reference) on the full workload (the bubble, the GCM, the LES or the
    bubble with hyperdiffusion; the oracle's elements in the GPU model's
    order): per-field relative L2 and max relative errors after one tendency
    evaluation and after `steps` LSRK54 steps from the same initial state,
    and the drift of total mass sum M rho and total energy sum M rho e
    (compensated sums, src/Arrays/MPIStateArrays.jl:655-675) over those
    steps.  Runs outside every timed region; independent of --steps."""
    import numpy as np

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    O.set_threads(os.cpu_count())
    om, _ = cpu_reference_case(O, workload)
    Q0 = np.ascontiguousarray(Q0, dtype=np.float64)
    M = dg64.grid.mass()
    t0 = time.perf_counter()
    ref_tend = om.tendency(Q0)
    Qo, _ = om.lsrk54(Q0.copy(), dt, steps)
    oracle_s = time.perf_counter() - t0
    sums0 = [om.weightedsum(Q0, f) for f in (0, 4)]
    sums_o = [om.weightedsum(Qo, f) for f in (0, 4)]
    rep = {"reference": "FP64 oracle (CPU restatement of the reference DGModel + LSRK54)", "steps": steps, "dt": dt,
           "oracle_seconds": oracle_s, "fields": ["rho", "rhou", "rhov", "rhow", "rhoe"]}
    drift = {"oracle": {"mass": (sums_o[0] - sums0[0]) / sums0[0], "energy": (sums_o[1] - sums0[1]) / sums0[1]}}
    for name, dg in (("mixed", dgmx), ("fp64", dg64)):
        Q = dg.init_ode_state(Q0)
        tend = dg.new_state(torch.float64)
        dg(tend, Q, None, 0.0)
        s_start = dg.weighted_sums(Q, (0, 4))
        lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
        cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=steps)
        s_end = dg.weighted_sums(Q, (0, 4))
        got = dg.full_state(Q).cpu().numpy()
        rep[name] = {"after_tendency": field_errors(tend.cpu().numpy(), ref_tend, M),
                     f"after_{steps}_steps": field_errors(got, Qo, M, base=Q0),
                     "status_word": dg.status_word()}
        drift[name] = {"mass": (s_end[0] - s_start[0]) / s_start[0], "energy": (s_end[1] - s_start[1]) / s_start[1]}
    rep["drift"] = drift
    rep["mixed_max_rel_l2"] = max(rep["mixed"][f"after_{steps}_steps"]["rel_l2"])
    rep["mixed_max_rel_l2_groups"] = max(rep["mixed"][f"after_{steps}_steps"]["rel_l2_rho_rhou_rhoe"])
    rep["target_rel_l2"] = 1e-5
    return rep


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="cmdg", choices=["cmdg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the accuracy report against the FP64 oracle (bubble, gcm, les, hyper)")
    ap.add_argument("--workload", default="bubble",
                    choices=["bubble", "bubble-arrays", "gcm", "les", "les16", "hyper", "ensemble", "hevi"])
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the batched-ensemble measurement the bubble line carries")
    ap.add_argument("--min-timed-s", type=float, default=MIN_TIMED_S,
                    help="each timed leg repeats its K-step region until it covers about this many seconds "
                         "(0: one region, as for a profiler run)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        # every requested step of the full workload, unless that would take
        # more than four minutes of host time (then as many as fit)
        r = run_cpu_reference(max(1, args.steps), warmup=args.warmup, max_sec=240.0)
        line = {"metric": "DOF-stage updates/s", "value": r["value"], "unit": "DOF-stage/s", "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": r["warmup"], "ms_per_step": 1e3 * r["sec"] / r["steps"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": WORKLOAD, "l2": L2_NOTE, "parallelism": f"replicas x{args.gpus}"},
                "run": {"path": "CPU FP64 oracle port of the reference DG + LSRK54"},
                "cpu_baseline": {"value": r["value"], "unit": "DOF-stage/s", "cores": r["threads"], "kind": "port",
                                 "sample": f"{r['steps']} timed LSRK54 steps (after {r['warmup']} warm-up) of the full 1e6-node workload"},
                "e2e": {"value": r["value"], "unit": "DOF-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import numpy as np
    import torch

    import __graft_entry__ as g

    g.build_library()
    import cmdg
    from cmdg import workloads

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    if args.workload == "ensemble":
        return bench_ensemble(args, cmdg, workloads, torch, barrier, stream, flush)
    if args.workload == "hevi":
        return bench_hevi(args, cmdg, workloads, torch, barrier, stream, flush)
    if args.workload == "les16":
        return bench_les16(args, cmdg, workloads, torch, barrier, stream, flush)

    spec = WORKLOADS[args.workload]

    def build(precision):
        if args.workload == "gcm":
            dg = workloads.gcm_shell_model(precision=precision)
            return dg, workloads.gcm_initial_state(dg.grid.coordinates())
        if args.workload == "les":
            dg = workloads.les_model(precision=precision)
            return dg, workloads.les_initial_state(dg.grid.coordinates())
        if args.workload == "bubble-arrays":
            dg, _, xyz = workloads.bubble_arrays_model(ne=NE, N=N, L=L, precision=precision)
            Q0 = workloads.rising_bubble(xyz, theta0=300.0, amp=2.0, rc=250.0, center=(1250.0, 1250.0, 350.0))
            return dg, Q0
        if args.workload == "hyper":
            dg = workloads.hyper_bubble_model(ne=NE, N=N, L=L, precision=precision)
        else:
            dg = workloads.bubble_model(ne=NE, N=N, L=L, precision=precision)
        xyz = dg.grid.coordinates()
        Q0 = workloads.rising_bubble(xyz, theta0=300.0, amp=2.0, rc=250.0, center=(1250.0, 1250.0, 350.0))
        return dg, Q0

    def n_repeats(step_ms):
        """How many times a leg repeats its timed region of exactly K steps so
        that the clock samples cover about MIN_TIMED_S of load (the same
        count on every rank)."""
        r = max(1, min(MAX_REPEATS, math.ceil(args.min_timed_s * 1e3 / max(step_ms * args.steps, 1e-3))))
        if dist is not None:
            t = torch.tensor([r], dtype=torch.int64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            r = int(t.item())
        return r

    def timed_run(dg, Q0, dt):
        """W warm-up steps, then R timed regions of exactly K steps, each
        starting from the initial state (copied in outside the timed region);
        returns the state after the last region (K steps from the initial
        state), the median region time, every step's time and R."""
        Q = dg.init_ode_state(Q0)
        Qinit = Q.clone()
        lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
        w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for i in range(max(args.warmup, 1)):
            if i == max(args.warmup, 1) - 1:
                w0.record(stream)
            cmdg.dostep_(Q, lsrk, None, 0.0)
        w1.record(stream)
        torch.cuda.synchronize()
        reps = n_repeats(w0.elapsed_time(w1))
        region_ms, per = [], []
        for r in range(reps):
            Q.copy_(Qinit)
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            barrier()
            for i in range(args.steps):
                flush.fill_(i & 0xFF)
                ev[i][0].record(stream)
                cmdg.dostep_(Q, lsrk, None, 0.0)
                ev[i][1].record(stream)
            barrier()
            ms = [a.elapsed_time(b) for a, b in ev]
            region_ms.append(sum(ms))
            per.extend(ms)
        return Q, statistics.median(region_ms), per, reps

    dg64, Q0 = build("fp64")
    dgmx, _ = build("mixed")
    kernels = {}
    for name, dg in (("fp64", dg64), ("mixed", dgmx)):
        kernels[name] = dg.autotune(reps=10)[1]
    dt = dg64.courant_dt(dg64.init_ode_state(Q0), CFL)
    nodes = dg64.grid.nelem * dg64.grid.Np

    clk = ClockSampler(local_rank).__enter__()  # sampled across the three timed legs
    Qmx, ms_mx, per_mx, reps_mx = timed_run(dgmx, Q0, dt)
    Q64, ms_64, per_64, reps_64 = timed_run(dg64, Q0, dt)

    # accuracy of the mixed path against the FP64 path after the last timed region's K steps
    a = dgmx.from_perturbation(Qmx).cpu().numpy()
    b = Q64.cpu().numpy()
    M = dg64.grid.mass()
    rel = [math.sqrt(float(np.sum((a[:, s] - b[:, s]) ** 2 * M))) / math.sqrt(float(np.sum(b[:, s] ** 2 * M)))
           for s in range(5)]
    # momentum as one vector field (a component that is nearly zero carries the others' rounding)
    rel_vec = [rel[0], math.sqrt(float(np.sum((a[:, 1:4] - b[:, 1:4]) ** 2 * M[:, None, :]))) /
               math.sqrt(float(np.sum(b[:, 1:4] ** 2 * M[:, None, :]))), rel[4]]

    # e2e: the FP64 state lives in pinned host memory; every step goes through
    # the C ABI's host-state entry point, which reads it over the host link,
    # steps, and writes the FP64 result back into host memory
    host = torch.from_numpy(np.ascontiguousarray(Q0)).pin_memory()
    Qp = dgmx.new_state(torch.float32)
    dQ = torch.zeros(host.shape, dtype=torch.float64, device="cuda")
    def e2e_step():
        dgmx.lsrk54_step_host(host, Qp, dQ, 0.0, dt, 1)

    host0 = host.clone()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(2):
        if i == 1:
            e0.record(stream)
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    reps_e2e = n_repeats(e0.elapsed_time(e1))
    e2e_ms = []
    for r in range(reps_e2e):
        host.copy_(host0)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        barrier()
        e2e_ms.append(e0.elapsed_time(e1))
    ms_e2e = statistics.median(e2e_ms)
    clk.__exit__(None, None, None)

    # max over ranks
    def rmax(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    ms_mx, ms_64, ms_e2e = rmax(ms_mx), rmax(ms_64), rmax(ms_e2e)
    work = world * NFIELD * nodes * NSTAGE * args.steps
    value = work / (ms_mx * 1e-3)
    v64 = work / (ms_64 * 1e-3)
    ve2e = work / (ms_e2e * 1e-3)
    peak, peak_kind = measured_peak()
    stage_ms_mx = ms_mx / args.steps / NSTAGE
    stage_ms_64 = ms_64 / args.steps / NSTAGE
    ach_mx = spec["bytes_mixed"] * nodes / (stage_ms_mx * 1e-3) / 1e9
    ach_64 = spec["bytes_fp64"] * nodes / (stage_ms_64 * 1e-3) / 1e9
    traffic = profile_traffic(spec["profile"])

    accuracy = None
    if rank == 0 and not args.no_accuracy and args.workload in ("bubble", "gcm", "les", "hyper"):
        try:
            accuracy = accuracy_report(cmdg, torch, dg64, dgmx, Q0, dt, workload=args.workload)
        except Exception as exc:  # the report must not hide the GPU line
            accuracy = {"error": str(exc)[:300]}

    ensemble = None
    if rank == 0 and not args.no_ensemble and args.workload == "bubble":
        try:
            # rank 0 alone: synchronise the device only (no collective barrier)
            ensemble = measure_ensemble(args, cmdg, workloads, torch, torch.cuda.synchronize, stream, flush)
        except Exception as exc:  # the ensemble leg must not hide the GPU line
            ensemble = {"error": str(exc)[:300]}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            r = run_cpu_reference(1, sample_steps=2, max_sec=60.0, workload=args.workload)
            cpu = {"value": r["value"], "unit": "DOF-stage/s", "cores": r["threads"], "kind": "port",
                   "sample": f"{r['steps']} LSRK54 steps (after {r['warmup']} warm-up) of the full "
                             f"{nodes:,}-node workload, FP64 oracle"}
        except Exception as exc:  # the CPU leg must not hide the GPU line
            cpu = {"value": None, "error": str(exc)[:200]}

    if rank == 0:
        line = {
            "metric": "DOF-stage updates/s", "value": value, "unit": "DOF-stage/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mx / args.steps,
            "node_stage_per_s": value / NFIELD,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": spec["desc"], "l2": L2_NOTE, "parallelism": f"replicas x{world}"},
            "run": {"path": "mixed FP32 perturbation / FP64 RK register", "dt": dt,
                    "stage_kernel": {k: list(v) for k, v in kernels.items()}},
            "fp64": {"value": v64, "ms_per_step": ms_64 / args.steps,
                     "roofline": {"bound": "hbm", "achieved": ach_64, "peak": peak, "unit": "GB/s",
                                  "frac": ach_64 / peak},
                     # the plain path is bound by the FP64 pipe (ncu capture of its stage kernel)
                     "fp64_pipe_frac": (profile_value("stage_kernel_fp64_bubble20.md", "fp64_pipe_frac")
                                        if args.workload == "bubble" else None),
                     "flops_per_node_stage": (profile_value("stage_kernel_fp64_bubble20.md",
                                                            "flops_per_node_stage_fp64")
                                              if args.workload == "bubble" else None)},
            "mixed_speedup_vs_fp64": value / v64,
            "mixed_step_ms": {"min": min(per_mx), "median": statistics.median(per_mx), "max": max(per_mx)},
            "mixed_vs_fp64_rel_l2": rel,
            "mixed_vs_fp64_rel_l2_rho_rhou_rhoe": rel_vec,
            "mixed_vs_fp64_steps": args.steps,
            # each leg times R regions of exactly K steps (restarting from the
            # initial state) and reports the median region
            "timed_regions": {"mixed": reps_mx, "fp64": reps_64, "e2e": reps_e2e},
            "accuracy": accuracy,
            # the batched mixed ensemble (the --workload ensemble measurement, same steps)
            "ensemble": ensemble,
            "roofline": {"bound": "hbm", "achieved": ach_mx, "peak": peak, "unit": "GB/s", "frac": ach_mx / peak,
                         "traffic": traffic, "peak_source": peak_kind,
                         "kernel": spec["kernel"], "bytes_per_node_stage": spec["bytes_mixed"],
                         # ncu FP instruction counts of the same kernel (profile summary)
                         "flops_per_node_stage": ({"fp32": profile_value(spec["profile"], "flops_per_node_stage_fp32"),
                                                   "fp64": profile_value(spec["profile"], "flops_per_node_stage_fp64")}
                                                  if args.workload == "bubble" else None)},
            "cpu_baseline": cpu,
            "e2e": {"value": ve2e, "unit": "DOF-stage/s", "h2d_bytes_per_step": int(host.numel() * 8),
                    "d2h_bytes_per_step": int(host.numel() * 8)},
            "gpu_launches": args.steps * NSTAGE * spec["launches_per_stage"],
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
