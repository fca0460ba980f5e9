#!/usr/bin/env python
"""Benchmark of the GB300 SBM hot path: 256^3 potential solve to rel-res 1e-8.

Workload (one "step" = one full solve): a 256^3 seeded synthetic
microstructure -- overlapping spheres, radii U[4,10] voxels, solid fraction
0.6, plus one random cylindrical tunnel of radius 6 -- whose signed distance
comes from 175 ReDist3D_XYZ steps and psi = 0.5(1 + tanh(d/(sqrt(2)*1.5))).
Node conductivity psi*1 + (1-psi)*0.1, Dirichlet phi = 0 / 1 on the two x
ghost planes, Neumann elsewhere, zero right-hand side; solved until
||r||/||r0|| <= 1e-8 (r recomputed in FP64).

Our arm (default): the production solver -- FP32 flexible CG with the
learned coarse-grid preconditioner (a 3D U-Net on the 4x-coarsened grid,
BF16 tcgen05 convolutions, weights elsim_gb300/weights/pc_unet.bin) applied
multiplicatively (coarse correction, then one Jacobi step with omega 2.3)
and FP64 reliable-update refinement -- with fields resident in HBM; `value`
is the mean device time of one solve (CUDA events on the solver stream),
`e2e` the same solve through the C-ABI from pinned host buffers
(coef/x/rhs uploaded, x downloaded) timed on the wall clock, the median of
at least 10 round trips (mean, extremes and samples beside it).  The plain FP64
CG (the drop-in), the FP32 Jacobi-PCG and the additive form of the learned
preconditioner are timed beside it (`--pc jacobi` makes Jacobi-PCG the
headline).

--impl reference: the reference's algorithm (plain FP64 CG, its own
restatement in C with OpenMP -- the Fortran reference has no compiler here)
timed on all host cores, each step a bounded sample of CG iterations
extrapolated to the 2038 iterations the FP64 CG needs on this workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 256
SEED = 1
TOL = 1e-8
METRIC = "sbm_potential_solve_time_256^3_relres_1e-8"
# dram__bytes_read.sum + dram__bytes_write.sum of one k32t_apply_dir launch
# at 256^3 (ncu): with the Jacobi read (Jacobi-PCG) and the flexible-CG
# variant of the learned preconditioner (7 words: z, p_old, hk, x read;
# p_new, q, x written).
APPLY_TRAFFIC = {1: 398.2e6, 2: 460.5e6}
# dram__bytes_read.sum + dram__bytes_write.sum of the 9 k_conv3_tc launches
# of one preconditioner application at 256^3 (ncu)
CONV_TRAFFIC = 41.56e6
UNIT = "s"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=N)
    ap.add_argument("--pc", default="learned", choices=["learned", "jacobi"],
                    help="preconditioner of the headline solve")
    ap.add_argument("--workload", default="solve256",
                    choices=["solve256", "batch96", "profile", "frontend", "step128", "unet64"],
                    help="solve256: the headline 256^3 solve; batch96: 96 uneven sub-volumes; "
                         "profile: only the production solve, for ncu captures; frontend: "
                         "one frame of the LevelSet_3D geometry front end; step128: the "
                         "full electrochemical time step at 128^3; unet64: forward passes "
                         "of the preconditioner's U-Net on the 64^3 coarse grid of a 256^3 "
                         "solve (the size its ncu captures use)")
    return ap.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _max_over_ranks(x: float, ws: int, device) -> float:
    """The largest of every rank's x (a job of replicas takes as long as
    its slowest one); x itself on one process."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _config(n, extra=None):
    cfg = {"workload": f"SBM potential solve {n}^3, spheres r~U[4,10] + tunnel r=6, "
                       f"solid 0.6, k=psi+0.1(1-psi), Dirichlet 0/1 on x faces, rel-res 1e-8",
           "grid": [n, n, n], "seed": SEED, "tol": TOL,
           "l2": "working set > L2 (>= 8 fields of 67-134 MB each) and an L2 flush "
                 "(256 MB write) between timed solves"}
    if extra:
        cfg.update(extra)
    return cfg


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi in the background."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        lines = [ln.strip() for ln in open(self.f.name) if ln.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
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
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("bf16_tflops_sustained", d.get("bf16_tflops"))), "measured (sustained)"
    return 1700.0, "fallback (sustained)"


# U-Net layers (cin, cout, level) of the learned preconditioner; level l has
# (n/4 / 2^l)^3 voxels on an n^3 grid
UNET = ((16, 16, 0), (16, 32, 1), (32, 32, 2), (32, 48, 3), (48, 64, 4),
        (112, 48, 3), (80, 32, 2), (64, 32, 1), (48, 16, 0))


def unet_flops(n):
    """2 x cin x cout x 27 x voxels summed over the 3x3x3 layers (the 1x1
    output layer is negligible)."""
    c = n // 4
    return sum(2 * ci * co * 27 * (c >> lev) ** 3 for ci, co, lev in UNET)


# --------------------------------------------------------------- CPU side

def _orc_threads(n):
    from oracle import sbm_oracle as orc
    orc.lib().orc_set_num_threads(n)
    return orc.lib().orc_num_threads()


def oracle_solve(prob, threads=0, tol=TOL, max_it=200000):
    """The reference's plain FP64 CG (the oracle's C restatement) run to
    convergence on `threads` host threads (0: all); returns (seconds, x,
    info).  Concentration problems carry their diagonal and scale."""
    from oracle import sbm_oracle as orc
    from elsim_gb300 import sbm
    used = _orc_threads(threads)
    try:
        bc = sbm.BC_COPY if "diag" in prob else sbm.BC_ZERO
        t = time.perf_counter()
        x, info = orc.cg(prob["coef"], prob["rhs"], prob["x"], prob.get("scale", 1.0), bc, bc,
                         sbm.STOP_REL_RES, tol, max_it, diag=prob.get("diag"))
        el = time.perf_counter() - t
    finally:
        _orc_threads(0)
    info["threads"] = used
    return el, x, info


def oracle_rate(prob, budget_s: float, full_iters: int, threads=0):
    """Oracle FP64 CG on `threads` host threads (0: all) for a bounded number
    of iterations (about budget_s seconds), scaled to `full_iters`, the
    iteration count a full solve of the same problem took (measured, not
    assumed); returns (seconds for the full solve, info)."""
    from oracle import sbm_oracle as orc
    from elsim_gb300 import sbm
    used = _orc_threads(threads)
    try:
        t = time.perf_counter()
        orc.cg(prob["coef"], prob["rhs"], prob["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
               sbm.STOP_REL_RES, 0.0, 3)
        per = (time.perf_counter() - t) / 3
        iters = int(max(3, min(full_iters, budget_s / max(per, 1e-6))))
        t = time.perf_counter()
        _, info = orc.cg(prob["coef"], prob["rhs"], prob["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
                         sbm.STOP_REL_RES, 0.0, iters)
        el = time.perf_counter() - t
    finally:
        _orc_threads(0)
    return el / info["iters"] * full_iters, {"iters": info["iters"], "seconds": el,
                                              "threads": used, "full_iters": full_iters}


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    from elsim_gb300 import synth
    from oracle import sbm_oracle as orc
    n = args.size
    m = synth.microstructure((n, n, n), seed=SEED, tunnel=True, redist=orc.redist)
    prob = synth.potential_problem(m["psi"])
    # one full solve first: it fixes the iteration count each bounded step
    # is scaled to, and its own time is reported beside the steps
    t_full, _, full = oracle_solve(prob)
    budget = 4.0
    for _ in range(args.warmup):
        oracle_rate(prob, budget / 4, full["iters"])
    vals, infos = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, info = oracle_rate(prob, budget, full["iters"])
        vals.append(v)
        infos.append(info)
    wall = time.perf_counter() - t0
    value = statistics.mean(vals)
    threads = infos[0]["threads"]
    sample = (f"{infos[0]['iters']} FP64 CG iterations of the {n}^3 solve per step on {threads} "
              f"OpenMP threads (oracle port of the reference CG), scaled to the {full['iters']} "
              f"iterations of a full oracle solve of the same problem measured in this run "
              f"({t_full:.2f} s)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded spheres + tunnel; reference inputs are not public)",
            "impl": "reference", "config": _config(n),
            "full_solve": {"s": t_full, "iterations": full["iters"], "threads": threads,
                           "final_rel_res": full["final_res"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------- GPU side

def concentration_solves(ctx, conc, pc, flush, reps=3):
    """The CnE-form concentration system (psE c - s div(psE grad c) = psE
    c_old, Neumann) of the headline microstructure on the same context:
    mixed-precision solves to rel-res TOL after one warm-up; returns (info,
    interior solution)."""
    import torch
    from elsim_gb300 import sbm
    for k in ("coef", "x", "rhs", "weight", "diag"):
        ctx.upload(k, conc[k])

    def solve():
        ctx.upload("x", conc["x"])
        flush.zero_()
        torch.cuda.synchronize()
        return ctx.cg_solve(op=sbm.OP_GENERIC_DIAG, bc_x0=sbm.BC_COPY, bc_x1=sbm.BC_COPY,
                            scale=conc["scale"], tol=TOL, max_it=200000,
                            stop_rule=sbm.STOP_REL_RES, precision=sbm.PREC_MIXED, precond=pc)

    solve()
    runs = [solve() for _ in range(reps)]
    x = ctx.download("x")[1:-1, 1:-1, 1:-1].copy()
    info = {"s": statistics.mean(r["ms"] for r in runs) / 1e3, "iterations": runs[-1]["iters"],
            "preconditioner": {0: "none", 1: "jacobi", 2: "learned"}.get(ctx.last_precond(), "?")}
    return info, x


def side_c1(net=None):
    """The plain 64^3 potential solve (spheres r ~ U[4,10], solid 0.6, 175
    reinitialisation steps, Dirichlet 0/1 on the x faces): GPU FP64 CG and
    the production mixed solve against the oracle's FP64 CG on all host
    threads and on one."""
    from elsim_gb300 import sbm, synth
    n1 = 64
    m1 = synth.microstructure((n1, n1, n1), seed=SEED)
    p1 = synth.potential_problem(m1["psi"])
    out = {"grid": [n1, n1, n1], "seed": SEED}
    with sbm.Context(n1, n1, n1) as c:
        for k in ("coef", "x", "rhs", "weight"):
            c.upload(k, p1[k])

        def sv(prec, pc):
            c.upload("x", p1["x"])
            return c.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO,
                              scale=1.0, tol=TOL, max_it=200000, stop_rule=sbm.STOP_REL_RES,
                              precision=prec, precond=pc)

        sv(sbm.PREC_FP64, sbm.PC_NONE)
        g64 = [sv(sbm.PREC_FP64, sbm.PC_NONE) for _ in range(3)]
        x_g = c.download("x")[1:-1, 1:-1, 1:-1].copy()
        x_l = None
        if net is not None:
            c.set_net(net)
            sv(sbm.PREC_MIXED, sbm.PC_LEARNED)
            gl = [sv(sbm.PREC_MIXED, sbm.PC_LEARNED) for _ in range(3)]
            x_l = c.download("x")[1:-1, 1:-1, 1:-1].copy()
            out["gpu_mixed_learned_s"] = statistics.mean(r["ms"] for r in gl) / 1e3
            out["gpu_mixed_learned_iterations"] = gl[-1]["iters"]
            out["gpu_mixed_learned_preconditioner"] = c.last_precond()
    t_all, xo, io = oracle_solve(p1)
    t_one, _, io1 = oracle_solve(p1, threads=1)
    xo = xo[1:-1, 1:-1, 1:-1]
    out.update({"gpu_fp64_cg_s": statistics.mean(r["ms"] for r in g64) / 1e3,
                "gpu_fp64_cg_iterations": g64[-1]["iters"],
                "cpu_fp64_cg_s": t_all, "cpu_threads": io["threads"],
                "cpu_fp64_cg_single_thread_s": t_one,
                "oracle_iterations": io["iters"],
                "relL2_fp64_cg_vs_oracle": float(np.linalg.norm(x_g - xo) / np.linalg.norm(xo))})
    if x_l is not None:
        out["relL2_mixed_learned_vs_oracle"] = float(np.linalg.norm(x_l - xo) / np.linalg.norm(xo))
    return out


def side_c2():
    """One full electrochemical time step at 128^3 (double-well
    Cahn-Hilliard, linearised Butler-Volmer, 20 reinitialisation steps): the
    GPU's device time for steps 2 and 3 of a run (step 1 skips the CnE
    solve) against the oracle's step 2 on all host threads and step 3 on one,
    and the GPU's fields after two steps against the oracle's."""
    import torch
    from elsim_gb300 import sbm, synth
    from oracle import sbm_oracle as orc
    shape = (128, 128, 128)
    p = synth.full_step_params(orc.params_reference())
    m2 = synth.microstructure(shape, seed=SEED, reinit_steps=20)
    d = m2["dist"][1:-1, 1:-1, 1:-1]
    dp, de = d.astype(np.float32), (-d).astype(np.float32)
    c0 = synth.full_step_concentration(shape, SEED)
    dt = synth.FULL_STEP_DT
    out = {"grid": list(shape), "seed": SEED}
    with sbm.Context(*shape, params=p) as ctx:
        s0 = ctx.setup_domain(dp, de)
        ctx.upload(sbm.F_CNP, c0)
        init = ctx.snapshot()
        vsr = synth.step_schedule(s0["xrf"], 0.0, s0["trgI"])[1]
        stream = torch.cuda.ExternalStream(ctx.stream())
        t2, t3 = [], []
        for rep in range(3):
            ctx.restore(init)
            ctx.time_step(1, dt, vsr)
            for it, acc in ((2, t2), (3, t3)):
                if it == 3 and rep == 2:
                    fields = {f: ctx.download(f) for f in (sbm.F_CNP, sbm.F_CNE, sbm.F_PHP,
                                                           sbm.F_PHE)}
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sc = ctx.time_step(it, dt, vsr)
                e1.record(stream)
                torch.cuda.synchronize()
                acc.append(e0.elapsed_time(e1) / 1e3)
                if it == 2:
                    s2 = sc
    st = orc.State(*shape, p)
    st.setup_domain(dp, de)
    st.set_field(sbm.F_CNP, c0)
    t = time.perf_counter()
    st.time_step(1, dt, vsr)
    t_o1 = time.perf_counter() - t
    t = time.perf_counter()
    so2 = st.time_step(2, dt, vsr)
    t_o2 = time.perf_counter() - t
    werr = {}
    for name, f, w in (("CnP", sbm.F_CNP, sbm.F_PSP), ("CnE", sbm.F_CNE, sbm.F_PSE),
                       ("phP", sbm.F_PHP, sbm.F_PSP), ("phE", sbm.F_PHE, sbm.F_PSE)):
        a, b = fields[f][1:-1, 1:-1, 1:-1], st.field(f)[1:-1, 1:-1, 1:-1]
        ww = st.field(w)[1:-1, 1:-1, 1:-1]
        werr[name] = float(np.sqrt((ww * (a - b) ** 2).sum() / max((ww * b * b).sum(), 1e-300)))
    threads = _orc_threads(1)
    try:
        t = time.perf_counter()
        st.time_step(3, dt, vsr)
        t_o3 = time.perf_counter() - t
    finally:
        _orc_threads(0)
    st.close()
    out.update({"gpu_step2_s": statistics.mean(t2), "gpu_step3_s": statistics.mean(t3),
                "cpu_step1_s": t_o1, "cpu_step2_s": t_o2,
                "cpu_threads": orc.lib().orc_num_threads(),
                "cpu_step3_single_thread_s": t_o3, "single_thread_check": threads,
                "weighted_rel_err_vs_oracle_after_2_steps": werr,
                "xrf_after_2_steps": {"gpu": s2["xrf"], "oracle": so2["xrf"]},
                "cg_iterations_step2": {"gpu": s2["it_cne"] + s2["it_php"] + s2["it_phe"],
                                        "oracle": so2["it_cne"] + so2["it_php"] + so2["it_phe"]}})
    return out


def run_ours(args):
    import torch
    ws, rank = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    from elsim_gb300 import sbm, synth

    n = args.size
    dev = torch.device("cuda", torch.cuda.current_device())
    m = synth.microstructure((n, n, n), seed=SEED, tunnel=True)
    prob = synth.potential_problem(m["psi"])
    hshape = prob["x"].shape
    nh = int(np.prod(hshape))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    ctx = sbm.Context(n, n, n)
    for k in ("coef", "x", "rhs", "weight"):
        ctx.upload(k, prob[k])

    def solve(prec, pc):
        ctx.upload("x", prob["x"])
        flush.zero_()
        torch.cuda.synchronize()
        return ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                            tol=TOL, max_it=200000, stop_rule=sbm.STOP_REL_RES, precision=prec,
                            precond=pc)

    head_pc = sbm.PC_LEARNED if args.pc == "learned" else sbm.PC_JACOBI
    net = None
    if head_pc == sbm.PC_LEARNED:
        from elsim_gb300 import learned
        net = learned.load()
        ctx.set_net(net)
    # the drop-in: plain FP64 CG (reference algorithm on the GPU)
    fp64 = solve(sbm.PREC_FP64, sbm.PC_NONE)
    x64 = ctx.download("x")[1:-1, 1:-1, 1:-1].copy()
    fp64_ms = ctx.bench_kernel(2, 10)
    plain = solve(sbm.PREC_MIXED, sbm.PC_NONE)
    # Jacobi-PCG beside the headline (same timing protocol)
    jac = [solve(sbm.PREC_MIXED, sbm.PC_JACOBI) for _ in range(max(1, args.warmup))]
    jac = [solve(sbm.PREC_MIXED, sbm.PC_JACOBI) for _ in range(max(1, args.steps))]
    jac_s = statistics.mean(r["ms"] for r in jac) / 1e3
    additive = None
    if head_pc == sbm.PC_LEARNED:
        # the learned preconditioner's additive form, for comparison
        ctx.set_tuning(pc_additive=True)
        solve(sbm.PREC_MIXED, head_pc)
        ad = [solve(sbm.PREC_MIXED, head_pc) for _ in range(max(1, args.steps))]
        additive = {"s": statistics.mean(r["ms"] for r in ad) / 1e3, "iterations": ad[-1]["iters"]}
        ctx.set_tuning(pc_additive=False)
    for _ in range(args.warmup):
        solve(sbm.PREC_MIXED, head_pc)
    # timed region: K solves, each timed on the device with CUDA events on the
    # solver stream (x reset and L2 flush happen between solves, untimed)
    clocks = Clocks()
    # a collection of the interpreter's garbage inside a timed solve stalls
    # the host that feeds the captured chunks (tens of ms with torch loaded)
    gc.collect()
    gc.disable()
    barrier()
    clocks.start()
    l0 = sbm.launch_count()
    t0 = time.perf_counter()
    times = []
    for _ in range(args.steps):
        info = solve(sbm.PREC_MIXED, head_pc)
        times.append(info["ms"] / 1e3)
    barrier()
    gc.enable()
    wall = time.perf_counter() - t0
    launches = sbm.launch_count() - l0
    clk = clocks.stop()
    used_pc = ctx.last_precond()
    xm = ctx.download("x")[1:-1, 1:-1, 1:-1]
    rel_err = float(np.linalg.norm(xm - x64) / np.linalg.norm(x64))
    t_local = _max_over_ranks(max(times), ws, dev)
    value = statistics.mean(times) if ws == 1 else t_local
    # kernel timings live on the solver stream: the fused direction + stencil
    # kernel (HBM roofline; the headline roofline for Jacobi-PCG) and, with
    # the learned preconditioner, its parts (the U-Net convolutions are the
    # dominant kernel of that solve: tensor roofline)
    ms_k, bytes_k = ctx.bench_kernel(0, 20)
    peak, peak_kind = _peaks()
    extra = {}
    roofline = None
    if used_pc == sbm.PC_LEARNED:
        ms_pc, bytes_pc = ctx.bench_kernel(3, 20)
        ms_cv, _ = ctx.bench_kernel(5, 20)
        ms_m, bytes_m = ctx.bench_kernel(6, 20)
        fl = unet_flops(n)
        tpk, tkind = _bf16_peak()
        extra["preconditioner_application"] = {
            "ms": ms_pc, "launches": 12, "fine_grid_GB/s": bytes_pc / (ms_pc * 1e-3) / 1e9,
            "unet_gflop": fl / 1e9,
            "unet_tflops_over_whole_application": fl / (ms_pc * 1e-3) / 1e12,
            "bf16_peak_tflops": tpk, "bf16_peak_kind": tkind,
            "note": "the convolutions are latency / shared-memory bound (small N, few CTAs on "
                    "the coarse levels), far from the tensor peak"}
        extra["multiplicative_step_kernel"] = {
            "kernel": "k_pc_mult_tiled (r -= alpha q, z = z1 + omega D^-1 (r - A z1), z.r, "
                      "z.q_old, r.r)", "ms": ms_m,
            "GB/s": bytes_m / (ms_m * 1e-3) / 1e9, "frac": bytes_m / (ms_m * 1e-3) / 1e9 / peak,
            "bound": "hbm"}
        # the dominant kernel of the solve (36 % of its time over 9 launches
        # per iteration): the U-Net convolutions on the tensor cores
        ach = fl / (ms_cv * 1e-3) / 1e12
        roofline = {"bound": "tensor", "kernel": "k_conv3_tc (the 9 U-Net convolutions of one "
                                                    "preconditioner application, BF16 tcgen05)",
                    "achieved": ach, "peak": tpk, "unit": "TFLOP/s", "frac": ach / tpk,
                    "peak_kind": tkind, "traffic": CONV_TRAFFIC, "algorithmic_flops": fl,
                    "ms": ms_cv}
    else:
        ms_u, bytes_u = ctx.bench_kernel(1, 20)
        extra["update_kernel"] = {"ms": ms_u, "GB/s": bytes_u / (ms_u * 1e-3) / 1e9}
    achieved = bytes_k / (ms_k * 1e-3) / 1e9
    apply_roofline = {"bound": "hbm", "kernel": "k32t_apply_dir (TMA-staged FP32 direction+stencil)"
                      + (", flexible-CG variant: no Jacobi read, the deferred x32 += alpha p_old "
                         "and R q in the same pass" if used_pc == sbm.PC_LEARNED else ""),
                      "achieved": achieved, "peak": peak, "unit": "GB/s",
                      "frac": achieved / peak, "peak_kind": peak_kind,
                      # DRAM read+write of one launch (ncu capture of the same variant)
                      "traffic": APPLY_TRAFFIC.get(used_pc),
                      "algorithmic_bytes": bytes_k, "ms": ms_k}
    # e2e through the C-ABI with pinned host buffers
    pin = {}
    for k in ("coef", "x", "rhs"):
        t = torch.empty(nh, dtype=torch.float64, pin_memory=True)
        a = np.ndarray(hshape, dtype=np.float64, buffer=t.numpy(), order="F")
        a[...] = prob[k]
        pin[k] = (t, a)
    xout_t = torch.empty(nh, dtype=torch.float64, pin_memory=True)
    e2e = []
    # W untimed warm-up round trips, then max(K, 10) timed ones: the host
    # side (a shared machine) varies by a few ms between round trips
    n_e2e = max(10, args.steps)
    gc.collect()
    gc.disable()
    for step in range(args.warmup + n_e2e):
        flush.zero_()
        barrier()
        t1 = time.perf_counter()
        for k in ("coef", "x", "rhs"):
            ctx.upload(k, pin[k][1])
        ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0, tol=TOL,
                     max_it=200000, stop_rule=sbm.STOP_REL_RES, precision=sbm.PREC_MIXED,
                     precond=head_pc)
        xo = np.ndarray(hshape, dtype=np.float64, buffer=xout_t.numpy(), order="F")
        lib = sbm.load_library()
        rc = lib.sbm_download(ctx._h, sbm.F_X, xo.ctypes.data_as(sbm.C.POINTER(sbm.C.c_double)), 1)
        assert rc == 0
        if step >= args.warmup:
            e2e.append(time.perf_counter() - t1)
    gc.enable()
    # the median: about one round trip in ten on the shared host stalls for
    # 15-19 ms on the host side (seen with the collector off too); the mean
    # and every sample stay in the line
    e2e_v = _max_over_ranks(statistics.median(e2e), ws, dev)
    cpu = None
    parity = {}
    side = {}
    if rank == 0 and ws == 1:
        # the concentration system of the same microstructure (CnE form)
        conc = synth.concentration_problem(m["psi"], SEED)
        cinfo, xc = concentration_solves(ctx, conc, head_pc, flush)
        # CPU legs: the reference's plain FP64 CG (oracle restatement) run to
        # convergence on all host threads -- its time is the like-for-like
        # baseline and its solution the parity reference -- and a bounded
        # single-thread sample scaled to the iteration count it measured
        t_full, xo, io = oracle_solve(prob)
        t_one, i_one = oracle_rate(prob, 10.0, io["iters"], threads=1)
        cpu = {"value": t_full, "unit": UNIT, "cores": io["threads"], "kind": "port",
               "sample": f"the whole {n}^3 solve: oracle FP64 CG (the reference's "
                         f"algorithm) to rel-res {TOL:g}, {io['iters']} iterations on "
                         f"{io['threads']} OpenMP threads",
               "iterations": io["iters"],
               "single_thread": {"value": t_one, "unit": UNIT, "cores": 1,
                                 "sample": f"{i_one['iters']} iterations on 1 thread "
                                           f"({i_one['seconds']:.1f} s), scaled to the "
                                           f"{io['iters']} iterations of the full solve"}}
        xo_i = xo[1:-1, 1:-1, 1:-1]
        t_oc, xoc, ioc = oracle_solve(conc)
        xoc_i = xoc[1:-1, 1:-1, 1:-1]
        parity = {
            "relL2_phi_vs_oracle": float(np.linalg.norm(xm - xo_i) / np.linalg.norm(xo_i)),
            "relL2_fp64_cg_vs_oracle": float(np.linalg.norm(x64 - xo_i) / np.linalg.norm(xo_i)),
            "oracle_iterations": io["iters"],
            "relL2_c_vs_oracle": float(np.linalg.norm(xc - xoc_i) / np.linalg.norm(xoc_i)),
            "concentration": {**cinfo, "oracle_s": t_oc, "oracle_iterations": ioc["iters"]},
            "like_for_like": {
                "what": "plain FP64 CG on the GPU (the drop-in) vs the same algorithm on the "
                        "host cores (oracle, all threads)",
                "gpu_fp64_cg_s": fp64["ms"] / 1e3, "cpu_fp64_cg_s": t_full,
                "speedup": t_full / (fp64["ms"] / 1e3)},
            "headline_vs_cpu_fp64_cg": t_full / value,
        }
        side = {"c1_plain_cg_64": side_c1(net if head_pc == sbm.PC_LEARNED else None),
                "c2_full_step_128": side_c2()}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" + ("+bf16" if used_pc == sbm.PC_LEARNED else ""),
            "data": "synthetic (seeded spheres + tunnel; reference inputs are not public)",
            "config": _config(n, {
                "method": ("FP32 flexible CG, learned U-Net coarse-grid correction (BF16 "
                           "tcgen05) followed by one Jacobi step (omega 2.3) on the remaining "
                           "residual, FP64 reliable-update refinement"
                           if used_pc == sbm.PC_LEARNED else
                           "FP32 Jacobi-PCG, FP64 reliable-update refinement"),
                "preconditioner": {0: "none", 1: "jacobi", 2: "learned"}.get(used_pc, "?"),
                "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                "iterations": info["iters"],
                "relL2_vs_fp64_cg": rel_err,
                "fp64_cg_s": fp64["ms"] / 1e3, "fp64_cg_iterations": fp64["iters"],
                "mixed_no_pc_s": plain["ms"] / 1e3, "mixed_no_pc_iterations": plain["iters"],
                "jacobi_pcg_s": jac_s, "jacobi_pcg_iterations": jac[-1]["iters"],
                "learned_additive_form": additive,
                "speedup_vs_fp64_cg": fp64["ms"] / 1e3 / value,
                "speedup_vs_jacobi_pcg": jac_s / value,
                "voxel_updates_per_s": n ** 3 * info["iters"] / value,
                "wall_s_timed_region": wall,
                **extra,
                "direction_stencil_kernel": apply_roofline,
                "fp64_stencil_kernel": {"ms": fp64_ms[0],
                                        "GB/s": fp64_ms[1] / (fp64_ms[0] * 1e-3) / 1e9,
                                        "bound": "fp64 alu"},
                **parity,
                **side,
            }),
            "roofline": roofline or apply_roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": 3 * nh * 8,
                    "d2h_bytes_per_step": nh * 8, "statistic": "median",
                    "round_trips": len(e2e), "mean": statistics.mean(e2e),
                    "min": min(e2e), "max": max(e2e),
                    "samples": [round(t, 6) for t in e2e]},
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line))
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batch(args):
    """96 independent sub-volumes, edges drawn from {48, 64, 96, 128}, one
    seed each, solid fraction U[0.5, 0.7]; per volume a potential system
    (GENERIC, Dirichlet 0/1 on the x faces) and a concentration system
    (GENERIC_DIAG: psE c - 0.1 div(psE grad c) = psE c_old, Neumann): all
    192 mixed-precision solves run to convergence in one CUDA-graph launch
    (one WHILE conditional node per system), launch shapes per edge length
    from the autotuner; the learned preconditioner (default) on every system
    it applies to (all potential systems; the concentration systems when the
    network reads the mass channel), Jacobi on the others.  Reports
    aggregate voxel-updates/s and each system's rel-L2 error against the
    oracle's FP64 CG solution."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from elsim_gb300 import autotune, sbm, synth
    rng = np.random.default_rng(2024)
    nv = 96
    edges = rng.choice([48, 64, 96, 128], size=nv)
    fracs = rng.uniform(0.5, 0.7, size=nv)
    probs, ctxs, ops, b0, b1, scales, kinds = [], [], [], [], [], [], []
    pc = sbm.PC_LEARNED if args.pc == "learned" else sbm.PC_JACOBI
    net = None
    if pc == sbm.PC_LEARNED:
        from elsim_gb300 import learned
        net = learned.load()
    for v in range(nv):
        n = int(edges[v])
        m = synth.microstructure((n, n, n), seed=5000 + v, solid_fraction=float(fracs[v]))
        for kind in ("potential", "concentration"):
            if kind == "potential":
                p = synth.potential_problem(m["psi"])
                ops.append(sbm.OP_GENERIC)
                b0.append(sbm.BC_ZERO)
                b1.append(sbm.BC_ZERO)
                scales.append(1.0)
            else:
                p = synth.concentration_problem(m["psi"], 5000 + v)
                ops.append(sbm.OP_GENERIC_DIAG)
                b0.append(sbm.BC_COPY)
                b1.append(sbm.BC_COPY)
                scales.append(p["scale"])
            c = sbm.Context(n, n, n)
            for k in ("coef", "x", "rhs", "weight", "diag"):
                if k in p:
                    c.upload(k, p[k])
            if net is not None:
                c.set_net(net)
            probs.append(p)
            ctxs.append(c)
            kinds.append(kind)
    tuned = {}
    for q, c in enumerate(ctxs):
        n = int(edges[q // 2])
        if kinds[q] != "potential":
            continue
        if n not in tuned:
            res = autotune.tune(c, lambda c=c, p=probs[q]: [c.upload(k, p[k]) for k in ("coef", "x", "rhs")])
            tuned[n] = res["best"]
    for c in ctxs:
        autotune.apply_cached(c)
    def reset():
        for c, p in zip(ctxs, probs):
            c.upload("x", p["x"])

    for _ in range(args.warmup):
        reset()
        sbm.batch_solve_ops(ctxs, ops, b0, b1, scales, tol=TOL, precond=pc)
    times, out = [], None
    l0 = sbm.launch_count()
    for _ in range(args.steps):
        reset()
        torch.cuda.synchronize()
        out = sbm.batch_solve_ops(ctxs, ops, b0, b1, scales, tol=TOL, precond=pc)
        times.append(out["ms"] / 1e3)
    launches = (sbm.launch_count() - l0) // max(1, args.steps)
    # every system's FP64 reference solution from the oracle (the reference's
    # plain CG, restated in C) on the host cores, to rel-res 1e-10
    errs = []
    t_oracle = 0.0
    for c, p in zip(ctxs, probs):
        t_o, xo, _ = oracle_solve(p, tol=1e-10)
        t_oracle += t_o
        xo = xo[1:-1, 1:-1, 1:-1]
        errs.append(float(np.linalg.norm(c.download("x")[1:-1, 1:-1, 1:-1] - xo)
                          / np.linalg.norm(xo)))
    t = statistics.mean(times)
    vu = sum(int(edges[q // 2]) ** 3 * out["iters"][q] for q in range(len(ctxs)))
    by = lambda kind: [e for e, k in zip(errs, kinds) if k == kind]
    its = lambda kind: [i for i, k in zip(out["iters"], kinds) if k == kind]
    line = {"metric": "sbm_batch96_solve_time", "value": t, "unit": "s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" + ("+bf16" if pc == sbm.PC_LEARNED else ""),
            "data": "synthetic (96 seeded sphere packings)",
            "config": {"workload": "96 sub-volumes, edges U{48,64,96,128}, solid U[0.5,0.7]; per "
                                   "volume a potential and a concentration system, rel-res "
                                   "1e-8, all 192 in one graph launch (a WHILE conditional node "
                                   "per system)",
                       "voxels": int(sum(int(e) ** 3 for e in edges)),
                       "systems": len(ctxs),
                       "max_relL2_vs_oracle": {"potential": max(by("potential")),
                                               "concentration": max(by("concentration"))},
                       "oracle_fp64_cg_s_all_systems": t_oracle,
                       "median_iterations": {"potential": float(np.median(its("potential"))),
                                             "concentration": float(np.median(its("concentration")))},
                       "all_converged": all(s_ == 0 for s_ in out["status"]),
                       "autotuned": {str(k): v for k, v in tuned.items()},
                       "voxel_updates_per_s": vu / t,
                       "preconditioner": {0: "none", 1: "jacobi", 2: "learned"}[pc],
                       "systems_with_learned_pc": {
                           k: sum(c.last_precond() == sbm.PC_LEARNED
                                  for c, kk in zip(ctxs, kinds) if kk == k)
                           for k in ("potential", "concentration")},
                       "batch_s": t},
            "gpu_launches": launches}
    print(json.dumps(line))
    for c in ctxs:
        c.close()
    return 0


def run_frontend(args):
    """One frame of the reference's geometry front end (LevelSet_3D.f90) at
    its own sizes: TmpA 500x520x170 (seeded synthetic 0/1 voxels in place of
    the scanned microstructure), grid 93 x 730 x 160, tunnel radius TuRd(8),
    50 Allen-Cahn steps, sign, 175 reinitialisation steps.  `value` = device
    time of a frame with the voxels resident; `e2e` = sbm_ls_frontend from
    pinned host buffers (voxels up, distance down); the oracle runs the same
    frame on the host cores and the two distances are compared bit for bit.
    `config.production_frame_s`: the same frame on the time-stepping
    program's 186 x 1460 x 320 grid (all lengths doubled)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from elsim_gb300 import geometry, sbm
    from oracle import sbm_oracle as orc
    R = geometry.REFERENCE
    yo, xo, zo, yg, zg, xoff, nth = (R[k] for k in ("yo", "xo", "zo", "yg", "zg", "xoff", "nthick"))
    xg = xoff + nth * zo
    n_fr = 8
    tr = float(geometry.TUNNEL_RADII[n_fr])
    ac, lit, dt = geometry.AC_ITERS, geometry.REDIST_ITERS, geometry.DT
    vox = geometry.synthetic_voxels((yo, xo, zo), seed=SEED)
    nv, nh = yo * xo * zo, (yg + 2) * (xg + 2) * (zg + 2)
    lib = sbm.load_library()
    dev = torch.device("cuda", 0)
    vox_d = torch.from_numpy(vox.ravel(order="F")).to(dev)
    ds, sg, tmp = (torch.empty(nh, dtype=torch.float64, device=dev) for _ in range(3))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def frame_dev(a=ac, n_lit=lit):
        sbm._check(lib.sbm_ls_frontend_device(vox_d.data_ptr(), yo, xo, zo, yg, zg, xoff, nth, tr,
                                              a, n_lit, dt, ds.data_ptr(), sg.data_ptr(),
                                              tmp.data_ptr(), stream.cuda_stream),
                   "sbm_ls_frontend_device")

    def timed(fn, k):
        out = []
        for _ in range(k):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1) / 1e3)
        return statistics.mean(out)

    for _ in range(args.warmup):
        frame_dev()
    torch.cuda.synchronize()
    clk = Clocks()
    clk.start()
    l0 = sbm.launch_count()
    t_frame = timed(frame_dev, args.steps)
    launches = (sbm.launch_count() - l0) // args.steps
    clocks = clk.stop()
    got = ds.cpu().numpy().reshape((yg + 2, xg + 2, zg + 2), order="F")
    t_nolit = timed(lambda: frame_dev(n_lit=0), args.steps)
    t_stack = timed(lambda: frame_dev(a=0, n_lit=0), args.steps)
    t_redist = (t_frame - t_nolit) / lit
    t_ac = (t_nolit - t_stack) / ac
    # end to end through the C-ABI from pinned host memory
    vox_h = torch.empty(nv, dtype=torch.float64, pin_memory=True)
    vox_h.numpy()[:] = vox.ravel(order="F")
    ds_h = torch.empty(nh, dtype=torch.float64, pin_memory=True)
    e2e = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sbm._check(lib.sbm_ls_frontend(C.cast(vox_h.data_ptr(), C.POINTER(C.c_double)), yo, xo, zo,
                                       yg, zg, xoff, nth, tr, ac, lit, dt,
                                       C.cast(ds_h.data_ptr(), C.POINTER(C.c_double))),
                   "sbm_ls_frontend")
        if i >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    # the production grid of the time-stepping program, 186 x 1460 x 320
    # (SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90:73-75): the same frame
    # with every length doubled (voxels upsampled 2x, 100 leading columns,
    # tunnel radius 2 TuRd(8)); device time of one frame after one warm-up
    del vox_d, ds, sg, tmp
    v2 = np.asfortranarray(np.repeat(np.repeat(np.repeat(vox, 2, 0), 2, 1), 2, 2))
    P = {"yo": 2 * yo, "xo": 2 * xo, "zo": 2 * zo, "yg": 2 * yg, "zg": 2 * zg, "xoff": 2 * xoff}
    xg2 = P["xoff"] + nth * P["zo"]
    nh2 = (P["yg"] + 2) * (xg2 + 2) * (P["zg"] + 2)
    v2_d = torch.from_numpy(v2.ravel(order="F")).to(dev)
    del v2
    b2 = [torch.empty(nh2, dtype=torch.float64, device=dev) for _ in range(3)]

    def frame_prod():
        sbm._check(lib.sbm_ls_frontend_device(v2_d.data_ptr(), P["yo"], P["xo"], P["zo"], P["yg"],
                                              P["zg"], P["xoff"], nth, 2 * tr, ac, lit, dt,
                                              b2[0].data_ptr(), b2[1].data_ptr(),
                                              b2[2].data_ptr(), stream.cuda_stream),
                   "sbm_ls_frontend_device")

    frame_prod()
    t_prod = timed(frame_prod, 2)
    del v2_d, b2
    # the AccDiff_3D program (1501 connectivity sweeps of each phase) on the
    # frame's distance, through the C-ABI (host psi, transfers included)
    dist = np.asfortranarray(got[1:-1, 1:-1, 1:-1])
    sbm.connectivity(dist, 0.75, 11)
    t0 = time.perf_counter()
    sbm.connectivity(dist, 0.75, 1501)
    t_conn = time.perf_counter() - t0
    # the oracle: the same frame on the host cores
    t0 = time.perf_counter()
    want = orc.ls_frontend(vox, yg, zg, xoff, nth, tr, ac, lit, dt)
    t_cpu = time.perf_counter() - t0
    threads = orc.lib().orc_num_threads()
    exact = bool(np.array_equal(got, want)) and bool(
        np.array_equal(ds_h.numpy().reshape(got.shape, order="F"), want))
    hbm, src = _peaks()
    redist_bytes = 3 * 8 * nh  # sg and f read, nf written, every padded cell
    ach = redist_bytes / t_redist / 1e9
    line = {"metric": "ls_frontend_frame_time_93x730x160", "value": t_frame, "unit": "s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_frame * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded thresholded smoothed noise, 60% ones; the scanned "
                    "microstructure is not public)",
            "config": {"workload": f"LevelSet_3D frame: TmpA {yo}x{xo}x{zo}, grid {yg}x{xg}x{zg}, "
                                   f"tunnel radius TuRd({n_fr}) = {tr:.4f}, {ac} Allen-Cahn + sign "
                                   f"+ {lit} ReDist3D steps",
                       "l2": "256 MB L2 flush between timed frames; working set 625 MB",
                       "bit_exact_vs_oracle": exact,
                       "ms_stack": t_stack * 1e3, "us_per_allen_cahn": t_ac * 1e6,
                       "us_per_redist": t_redist * 1e6,
                       "production_grid": f"{2 * yg}x{xg2}x{2 * zg} (lengths x2, voxels "
                                          f"{2 * yo}x{2 * xo}x{2 * zo})",
                       "production_frame_s": t_prod,
                       "connectivity_program_s": t_conn},
            "roofline": {"kernel": "k_redist", "bound": "hbm", "achieved": ach, "peak": hbm,
                         "unit": "GB/s", "frac": ach / hbm, "peak_source": src,
                         "traffic": None,
                         "note": "FP64-pipe-bound on GB300; algorithmic bytes 24 B x "
                                 f"{nh} padded cells per launch"},
            "cpu_baseline": {"value": t_cpu, "unit": "s", "cores": threads, "kind": "port",
                             "sample": "the whole frame (oracle C restatement, OpenMP)"},
            "e2e": {"value": statistics.mean(e2e), "unit": "s", "h2d_bytes_per_step": 8 * nv,
                    "d2h_bytes_per_step": 8 * nh},
            "clocks": clocks, "gpu_launches": launches}
    print(json.dumps(line))
    return 0


def run_step128(args):
    """The full electrochemical step at 128^3 (double-well Cahn-Hilliard,
    linearised Butler-Volmer with i0 = 1e-3, 20 reinitialisation steps,
    c0 = 0.5 +- 0.01, dt = 1e-3): `steps` x 100 time steps on the GPU after
    `warmup` x 10; `value` = device time per time step (CUDA events on the
    context stream).  The oracle runs the first two steps of the same run on
    the host cores (CPU baseline per step), and the GPU's fields after them
    are compared with the oracle's."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from elsim_gb300 import sbm, synth
    from oracle import sbm_oracle as orc
    n = 128
    shape = (n, n, n)
    p = synth.full_step_params(orc.params_reference())
    m = synth.microstructure(shape, seed=SEED, reinit_steps=20)
    d = m["dist"][1:-1, 1:-1, 1:-1]
    dp, de = d.astype(np.float32), (-d).astype(np.float32)
    c0 = synth.full_step_concentration(shape, SEED)
    dt = synth.FULL_STEP_DT
    ctx = sbm.Context(*shape, params=p)
    s0 = ctx.setup_domain(dp, de)
    ctx.upload(sbm.F_CNP, c0)
    init = ctx.snapshot()
    vsr = synth.step_schedule(s0["xrf"], 0.0, s0["trgI"])[1]
    stream = torch.cuda.ExternalStream(ctx.stream())
    nsteps = 100

    def run(k):
        hist = []
        for it in range(1, k + 1):
            hist.append(ctx.time_step(it, dt, vsr))
        return hist

    for _ in range(args.warmup):
        ctx.restore(init)
        run(10)
    times, iters = [], []
    clk = Clocks()
    clk.start()
    l0 = sbm.launch_count()
    for _ in range(args.steps):
        ctx.restore(init)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        hist = run(nsteps)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3 / nsteps)
        iters.append(sum(h["it_cne"] + h["it_php"] + h["it_phe"] for h in hist))
    launches = (sbm.launch_count() - l0) // args.steps
    clocks = clk.stop()
    # the oracle: the first two steps of the same run, then the GPU's fields
    ctx.restore(init)
    g2 = run(2)
    st = orc.State(*shape, p)
    so = st.setup_domain(dp, de)
    st.set_field(sbm.F_CNP, c0)
    t0 = time.perf_counter()
    for it in (1, 2):
        so = st.time_step(it, dt, vsr)
    t_cpu = (time.perf_counter() - t0) / 2
    werr = {}
    for name, f, w in (("CnP", sbm.F_CNP, sbm.F_PSP), ("CnE", sbm.F_CNE, sbm.F_PSE),
                       ("phP", sbm.F_PHP, sbm.F_PSP), ("phE", sbm.F_PHE, sbm.F_PSE)):
        a, b, ww = ctx.download(f)[1:-1, 1:-1, 1:-1], st.field(f)[1:-1, 1:-1, 1:-1], \
            st.field(w)[1:-1, 1:-1, 1:-1]
        werr[name] = float(np.sqrt((ww * (a - b) ** 2).sum() / max((ww * b * b).sum(), 1e-300)))
    threads = orc.lib().orc_num_threads()
    t = statistics.mean(times)
    line = {"metric": "sbm_full_step_time_128^3", "value": t, "unit": "s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded spheres, 20 reinitialisation steps)",
            "config": {"workload": "full electrochemical time step 128^3: double-well CH (W=1, "
                                   "kappa=1 voxel^2, M=1), linearised BV i0=1e-3, dt=1e-3, "
                                   "c0=0.5+-0.01; one step = CH, CnE solve, BV Picard with phP "
                                   "/ phE solves, voltage control",
                       "time_steps_per_run": nsteps, "cg_iterations_per_run": iters[-1],
                       "xrf_after": hist[-1]["xrf"],
                       "weighted_rel_err_vs_oracle_after_2_steps": werr,
                       "xrf_after_2_steps": {"gpu": g2[-1]["xrf"], "oracle": so["xrf"]}},
            "cpu_baseline": {"value": t_cpu, "unit": "s", "cores": threads, "kind": "port",
                             "sample": "time steps 1-2 of the same run (oracle C restatement, "
                                       "OpenMP)"},
            "clocks": clocks, "gpu_launches": launches}
    print(json.dumps(line))
    ctx.close()
    return 0


def run_profile(args):
    """The production solve alone (no FP64 baseline, no CPU leg), `steps`
    times after `warmup` solves: the command the ncu summaries profile.  Its
    iteration chunks are driven from the host (the same kernels): ncu does
    not profile kernels inside the conditional graph that loops them on the
    device."""
    import __graft_entry__
    __graft_entry__.build()
    from elsim_gb300 import sbm, synth
    n = args.size
    m = synth.microstructure((n, n, n), seed=SEED, tunnel=True)
    prob = synth.potential_problem(m["psi"])
    pc = sbm.PC_LEARNED if args.pc == "learned" else sbm.PC_JACOBI
    with sbm.Context(n, n, n) as ctx:
        for k in ("coef", "x", "rhs", "weight"):
            ctx.upload(k, prob[k])
        ctx.set_tuning(host_loop=True)
        if pc == sbm.PC_LEARNED:
            from elsim_gb300 import learned
            net = learned.load()
            ctx.set_net(net)
        for _ in range(args.warmup + args.steps):
            ctx.upload("x", prob["x"])
            info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO,
                                scale=1.0, tol=TOL, max_it=200000, stop_rule=sbm.STOP_REL_RES,
                                precision=sbm.PREC_MIXED, precond=pc)
        print(json.dumps({"workload": "profile", "n": n, **info}))
    return 0


def run_unet64(args):
    """Forward passes of the learned preconditioner's U-Net (stored weights)
    on the 64^3 coarse grid of a 256^3 solve, through sbm_net_forward (host
    input, uploaded once per call): `steps` calls after `warmup`; `value` =
    wall time per call, the tensor roofline of the convolutions from the
    same FLOP count as the headline line."""
    import __graft_entry__
    __graft_entry__.build()
    from elsim_gb300 import learned
    net = learned.load()
    rng = np.random.default_rng(SEED)
    c = 64
    x = rng.normal(size=(c ** 3, 16)).astype(np.float32)
    x[:, 5:] = 0.0
    x[:, 2] = 1.0
    for _ in range(args.warmup):
        net.forward(x, (c, c, c))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = net.forward(x, (c, c, c))
    t = (time.perf_counter() - t0) / args.steps
    print(json.dumps({"workload": "unet64", "coarse_grid": [c, c, c], "s_per_call": t,
                      "unet_gflop": unet_flops(4 * c) / 1e9, "out_rms": float(np.sqrt((out ** 2).mean()))}))
    return 0


def main():
    args = _args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch96":
        return run_batch(args)
    if args.workload == "profile":
        return run_profile(args)
    if args.workload == "frontend":
        return run_frontend(args)
    if args.workload == "step128":
        return run_step128(args)
    if args.workload == "unet64":
        return run_unet64(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
