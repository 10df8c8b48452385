#!/usr/bin/env python
"""Benchmark: time to ||R||/||R0|| < 1e-8 on every load step of one load path (20 LoadControl steps) on the
128x32x32 jittered Q1 Neo-Hooke cantilever (131072 elements, 421443 dofs), mixed-precision form
(FP32 tangent / FP32 block-Jacobi CG, FP64 residual, Eisenstat-Walker inexact Newton) against the plain FP64
GPU form (FP64 tangent, FP64 block-Jacobi CG to 1e-10), plus the roofline of the dominant kernel (the CG SpMV).

A step = one complete load path from the undeformed state.  `value` is device time per load path with the
inputs resident in HBM; `e2e` adds the host->device copy of the initial displacement and the device->host
copy of the converged displacement, through the public API.  Prints one JSON line.  Beside the headline the
line carries `two_level`: the same load path with the CG's coarse correction (an additive two-level
preconditioner, `--coarse` slabs; not the headline's block-Jacobi method), both forms.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to ||R||/||R0||<1e-8 per load path (mixed vs plain FP64 GPU)"


def max_over_ranks(value: float, world: int, device="cuda") -> float:
    """The slowest rank's value (replicas: every rank times its own copy of the workload); plain value at N = 1.
    The all-reduce runs on `device` ("cuda" under NCCL, "cpu" under gloo)."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--load-steps", type=int, default=20)
    ap.add_argument("--plain-runs", type=int, default=1)
    ap.add_argument("--eta-max", type=float, default=2e-2, help="mixed form: Eisenstat-Walker forcing upper bound")
    ap.add_argument("--eta-min", type=float, default=1e-5, help="mixed form: Eisenstat-Walker forcing lower bound")
    ap.add_argument("--predictor", type=int, default=1, choices=[0, 1, 3],
                    help="mixed form's Newton predictor: 0 none (the reference's), 1 previous increment (the learned "
                         "predictor's fallback; this single load case has no trained model), 3 second-order "
                         "extrapolation with the previous increment as fallback")
    ap.add_argument("--coarse", type=int, default=16,
                    help="slabs of the CG's coarse correction for the extra two-level measurement beside the "
                         "headline (0: skip it)")
    ap.add_argument("--tangent-kernel", type=int, default=0, choices=[0, 1, 2, 3],
                    help="mixed form's FP32 tangent kernel: 0 timed choice, 1 coloured, 2 row, 3 element blocks")
    ap.add_argument("--coarse-refresh", type=int, default=4,
                    help="two-level measurement: rebuild A_c at every n-th factorize (1: every one)")
    ap.add_argument("--two-level-only", action="store_true",
                    help="only the two-level measurement (mixed and plain FP64 with the coarse correction)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cg-kernel", default="",
                    help="mixed form's CG kernel as kind[:keep] (default: the autotuner's choice)")
    ap.add_argument("--ref-budget", type=float, default=240.0,
                    help="--impl reference: seconds after which no further load step is started (at least one runs)")
    ap.add_argument("--small", action="store_true", help="32x8x8 mesh (profiling runs)")
    ap.add_argument("--config", type=int, default=2, choices=[2, 3, 4, 5],
                    help="2: 128x32x32 cantilever (default, the headline); 3: 512 batched cantilevers; "
                         "4: learned predictor on 64x16x16; 5: nearly incompressible EAS block")
    ap.add_argument("--train-paths", type=int, default=200, help="config 4: training load paths")
    ap.add_argument("--eval-paths", type=int, default=20, help="config 4: held-out load paths")
    ap.add_argument("--no-graphs", action="store_true", help="launch CG kernels one by one (for profilers)")
    ap.add_argument("--batched-eta-max", type=float, default=1e-2,
                    help="config 3: mixed form's Eisenstat-Walker upper bound (linear tolerance of the first iteration)")
    ap.add_argument("--batched-trace", action="store_true",
                    help="config 3: only the mixed and plain forms, with a per-Newton-iteration trace (wall time, "
                         "largest per-instance CG count) summarised in the line")
    ap.add_argument("--batched-backtracks", type=int, default=8,
                    help="config 3: halvings of an instance's correction that inverts an element (0: take it out)")
    ap.add_argument("--backtracks", type=int, default=0,
                    help="configs 3 and 5: halve a Newton correction that inverts an element up to this many times "
                         "(both forms; 0 = abort like the reference)")
    ap.add_argument("--eas-cg-cap", type=int, default=5000,
                    help="config 5, mixed form: CG iterations per Newton step at most (an FP32 CG on the nearly "
                         "incompressible tangent stagnates; the Newton step goes on with the capped iterate)")
    ap.add_argument("--eas-restart", type=int, default=20,
                    help="config 5: restart length of the mixed form's FP64 outer GMRES (0: FP32 CG alone)")
    ap.add_argument("--eas-inner-rtol", type=float, default=1e-2,
                    help="config 5: relative tolerance of the FP32 CG inside the FP64 outer solve")
    ap.add_argument("--eas-size", default="64,64,16", help="config 5: elements per direction")
    ap.add_argument("--eas-steps", type=int, default=25, help="config 5: load steps")
    ap.add_argument("--eas-first-steps", type=int, default=0,
                    help="config 5: run only the first K of the load steps (a short run for profiling; 0 = all)")
    ap.add_argument("--eas-predictor", type=int, default=1, help="config 5: 0 none, 1 previous increment")
    ap.add_argument("--path-following", type=int, default=0,
                    help="arc-length path of this many steps on the 128x32x32 cantilever instead of the load control")
    ap.add_argument("--pf-mixed-only", action="store_true", help="--path-following: skip the plain FP64 form")
    ap.add_argument("--no-warm-start", action="store_true",
                    help="--path-following: start the load column's CG from zero in every Newton iteration")
    ap.add_argument("--no-multi-rhs", action="store_true",
                    help="--path-following: solve the two bordered columns one after the other")
    ap.add_argument("--spmv-kinds", default="-1", help="--spmv-only: comma-separated kind[:keep] SpMV choices")
    ap.add_argument("--spmv-precision", type=int, default=1, help="--spmv-only: 1 FP32 tangent, 0 FP64")
    ap.add_argument("--spmv-only", type=int, default=0,
                    help="assemble the 128x32x32 tangent once (FP32) and run this many CG iterations, then exit "
                         "(the case the SpMV ncu captures run)")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows, self.proc, self.gpu = [], None, gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def log(msg):
    print(msg, file=sys.stderr, flush=True)


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------------------------------------
def solver_settings(ikr, mixed: bool, eta=(2e-2, 1e-5)):
    if mixed:
        return ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=eta[0],
                              linear_rtol_min=eta[1], linear_max_iter=200000)
    return ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, linear_rtol=1e-10, linear_max_iter=400000)


class Form:
    """One solution form (mixed or plain) on the GPU: element set, assembler, solver objects, requirements."""

    def __init__(self, ikr, problems, p, mixed, predictor=0, eta=(1e-2, 1e-5), coarse=0, coarse_refresh=1):
        self.ikr = ikr
        self.mixed = mixed
        self.fes, self.asm = problems.build_gpu(p, precision=1 if mixed else 0)
        self.ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi)
        if coarse:
            self.ls.set_coarse_space(coarse)
            self.ls.set_coarse_refresh(coarse_refresh)
        self.nr = ikr.NewtonRaphson(self.asm, ikr.NewtonRaphsonConfig(solver_settings(ikr, mixed, eta), self.ls))
        self.lc = ikr.LoadControl(self.nr, p.load_steps, (0.0, p.t_end))
        if predictor:
            self.lc.set_predictor(predictor)
        self.req = ikr.FERequirements(self.fes)
        self.req0 = ikr.FERequirements(self.fes)  # undeformed state, load factor 0 (device resident)
        self.asm.bind(self.req, ikr.DBCOption.Full)

    def run_device(self):
        self.req.assign(self.req0)
        return self.lc.run(self.req)


def make_events(torch, stream_ptr):
    st = torch.cuda.ExternalStream(stream_ptr)
    return st, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def spmv_bytes(asm, n_nodes, value_bytes):
    """Algorithmic bytes of one fused CG SpMV launch: values + column indices + row pointers of the 3x3-block
    matrix, and the four dof vectors it streams (z, p_old read; p_new, q written)."""
    rp, col = asm.block_pattern()
    nb = len(col)
    n = 3 * n_nodes
    return nb * (9 * value_bytes + 4) + 4 * (n_nodes + 1) + 4 * n * value_bytes, nb


def run_ours(args, rank, world):
    import numpy as np
    import torch

    import ikarus_gb300 as ikr
    from ikarus_gb300 import problems

    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    p = problems.cantilever(32, 8, 8, jitter=0.1, seed=2024, load_steps=args.load_steps, tol=1e-8, relative=True) \
        if args.small else problems.config2(load_steps=args.load_steps)
    n_nodes = p.mesh.n_nodes
    mixed = Form(ikr, problems, p, mixed=True, predictor=args.predictor, eta=(args.eta_max, args.eta_min))
    if args.cg_kernel:
        kind, _, keep = args.cg_kernel.partition(":")
        mixed.ls.set_kernel(int(kind), float(keep) if keep else -1.0)
    if args.tangent_kernel:
        mixed.asm.set_tangent_kernel(args.tangent_kernel)
    stream, ev0, ev1 = make_events(torch, mixed.fes.stream())
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # warm-up
    for _ in range(args.warmup):
        t0 = time.perf_counter()
        info = mixed.run_device()
        log(f"warmup mixed: {time.perf_counter() - t0:.3f} s, newton {info.totalIterations}, "
            f"cg {info.totalLinearIterations}, ok {info.success}")
        assert info.success, "mixed-precision load path failed"
    barrier()

    # timed: device-resident inputs
    times, infos = [], []
    launches0 = ikr.kernel_launches()
    local_gpu = 0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank))
    with ClockSampler(local_gpu) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            mixed.req.assign(mixed.req0)
            torch.cuda.synchronize()
            ev0.record(stream)
            info = mixed.lc.run(mixed.req)
            ev1.record(stream)
            ev1.synchronize()
            times.append(ev0.elapsed_time(ev1) / 1e3)
            infos.append(info)
        barrier()
    launches = (ikr.kernel_launches() - launches0) // max(1, args.steps)
    # one more (untimed) load path with device events around every CG SpMV inside the graphs: the dominant
    # kernel's average duration for the roofline (the event nodes would perturb the timed region)
    mixed.ls.profile(True)
    flush.zero_()
    torch.cuda.synchronize()
    pinfo = mixed.run_device()
    assert pinfo.success
    spmv_ms, spmv_n = mixed.ls.profile_read()
    prof_solves = pinfo.totalIterations  # one CG solve per Newton iteration (no refinement sweeps in this form)
    mixed.ls.profile(False)
    assembly = {"mixed": assembly_rates(ikr, torch, mixed, p)}
    assert all(i.success for i in infos)
    t_mixed = max_over_ranks(sum(times) / len(times), world)

    # e2e: public API with host buffers (h2d initial displacement, d2h converged displacement)
    u0 = np.zeros(p.n_dofs)
    e2e = []
    for _ in range(min(args.steps, 2)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mixed.req.insertGlobalSolution(u0)
        mixed.req.insertParameter(0.0)
        info = mixed.lc.run(mixed.req)
        u = mixed.req.globalSolution()
        e2e.append(time.perf_counter() - t0)
        assert info.success and np.isfinite(u).all()
    t_e2e = sum(e2e) / len(e2e)

    # plain FP64 form of the same method
    del flush
    if args.plain_runs <= 0:
        return finish(args, p, world, t_mixed, t_e2e, None, None, infos, launches, mixed, n_nodes, spmv_ms, spmv_n,
                      clocks, None, prof_solves, assembly), p
    plain = Form(ikr, problems, p, mixed=False)
    pstream, pev0, pev1 = make_events(torch, plain.fes.stream())
    plain_times, plain_infos = [], []
    for _ in range(args.plain_runs):
        plain.req.assign(plain.req0)
        torch.cuda.synchronize()
        pev0.record(pstream)
        pinfo = plain.lc.run(plain.req)
        pev1.record(pstream)
        pev1.synchronize()
        plain_times.append(pev0.elapsed_time(pev1) / 1e3)
        plain_infos.append(pinfo)
        log(f"plain fp64: {plain_times[-1]:.3f} s, newton {pinfo.totalIterations}, cg {pinfo.totalLinearIterations}")
    t_plain = sum(plain_times) / len(plain_times)
    u_plain = plain.req.globalSolution()
    u_mixed = mixed.req.globalSolution()
    rel_diff = float(np.abs(u_mixed - u_plain).max() / np.abs(u_plain).max())
    assembly["plain_fp64"] = assembly_rates(ikr, torch, plain, p)
    out = finish(args, p, world, t_mixed, t_e2e, t_plain, plain_infos[-1], infos, launches, mixed, n_nodes, spmv_ms,
                 spmv_n, clocks, rel_diff, prof_solves, assembly)
    del plain, mixed
    if args.coarse > 0:
        out["two_level"] = run_two_level(args, ikr, torch, problems, p, u_plain, t_plain)
    return out, p


def run_two_level(args, ikr, torch, problems, p, u_plain, t_plain_bj):
    """Not the headline (whose method is block-Jacobi PCG): the same load path with the CG's coarse correction
    (LinearSolver.set_coarse_space, an additive two-level preconditioner with the rigid-body modes of
    `args.coarse` slabs), mixed form (one untimed and two timed paths) and plain FP64 form (one path), device
    time with the same 256 MB L2 flush before each path."""
    import numpy as np

    res = {"slabs": args.coarse, "coarse_refresh": args.coarse_refresh,
           "preconditioner": "block Jacobi + P A_c^-1 P^T (six rigid-body modes per slab, A_c = P^T K P rebuilt at "
                             "every coarse_refresh-th factorize)"}
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    try:
        for key, mixed, runs in (("mixed", True, 3), ("plain_fp64", False, 1)):
            f = Form(ikr, problems, p, mixed=mixed, predictor=args.predictor if mixed else 0,
                     eta=(args.eta_max, args.eta_min), coarse=args.coarse, coarse_refresh=args.coarse_refresh)
            st, e0, e1 = make_events(torch, f.fes.stream())
            times = []
            for k in range(runs):
                f.req.assign(f.req0)
                flush.zero_()
                torch.cuda.synchronize()
                e0.record(st)
                info = f.lc.run(f.req)
                e1.record(st)
                e1.synchronize()
                assert info.success, f"two-level {key} load path failed"
                if not mixed or k > 0:
                    times.append(e0.elapsed_time(e1) / 1e3)
                log(f"two-level {key}: {e0.elapsed_time(e1) / 1e3:.3f} s, newton {info.totalIterations}, "
                    f"cg {info.totalLinearIterations}, {f.ls.coarse_info()}")
            u = f.req.globalSolution()
            if mixed:  # cost split on the last tangent: factorize (with A_c) and CG iterations, with and without
                b = np.where(p.fixed == 1, 0.0, 1.0)
                split = {}
                for slabs in (args.coarse, 0):
                    ls2 = ikr.LinearSolver(rtol=1e-5, max_iter=20000)
                    ls2.set_coarse_space(slabs)
                    ls2.compute(f.asm)  # the kind is tuned here
                    ls2.solve(f.asm, b)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    ls2.compute(f.asm)
                    torch.cuda.synchronize()
                    t1 = time.perf_counter()
                    ls2.solve(f.asm, b)
                    t2 = time.perf_counter()
                    it, _ = ls2.last_info()
                    split["with_coarse" if slabs else "block_jacobi_two_kernel"] = {
                        "factorize_ms": round(1e3 * (t1 - t0), 3), "cg_iterations_to_1e-5": it,
                        "us_per_cg_iteration": round(1e6 * (t2 - t1) / max(it, 1), 2), "kind": ls2.kernel_info()[:2]}
                    del ls2
                res["cost_split_fp32_last_tangent"] = split
            res[key] = {"s_per_load_path": round(sum(times) / len(times), 4), "newton_iterations": info.totalIterations,
                        "cg_iterations": info.totalLinearIterations, "spmv_kernel": f.ls.kernel_info()[:2],
                        "max_rel_diff_vs_plain_block_jacobi": None if u_plain is None else
                        float(np.abs(u - u_plain).max() / np.abs(u_plain).max()),
                        **f.ls.coarse_info()}
            del f
        res["speedup_mixed_vs_plain_fp64_both_two_level"] = round(res["plain_fp64"]["s_per_load_path"]
                                                                   / res["mixed"]["s_per_load_path"], 2)
        if t_plain_bj:
            res["speedup_vs_plain_fp64_block_jacobi"] = round(t_plain_bj / res["mixed"]["s_per_load_path"], 2)
    except Exception as e:  # reported, the headline stands on its own
        res["failed"] = f"{type(e).__name__}: {e}"
    return res


def assembly_rates(ikr, torch, form, p):
    """Device time of one residual assembly (FP64) and one tangent assembly (the form's precision) at the form's
    current state, averaged over 5 after a warm-up: elements/s, dofs/s and achieved bytes/s of the algorithmic
    traffic (values written once, coordinates, displacements, connectivity and the element-to-block map read
    once; residual written once)."""
    stream, e0, e1 = make_events(torch, form.fes.stream())
    out = {}
    nn, ne, n = p.mesh.n_nodes, p.mesh.n_elems, p.n_dofs
    rp, col = form.asm.block_pattern()
    nb = len(col)
    sK = 4 if form.mixed else 8
    common = nn * 3 * 8 + n * 8 + ne * 8 * 4
    for name, call, nbytes in (
            ("residual_fp64", lambda: form.asm.vector(form.req, dbc=ikr.DBCOption.Full, export=False),
             common + n * 8),
            ("tangent_fp32" if form.mixed else "tangent_fp64",
             lambda: form.asm.matrix(form.req, dbc=ikr.DBCOption.Full, export=False),
             common + nb * 9 * sK + ne * 64 * 4)):
        call()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(5):
            call()
        e1.record(stream)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 5 / 1e3
        out[name] = {"ms": round(t * 1e3, 3), "elements_per_s": round(ne / t), "dofs_per_s": round(n / t),
                     "algorithmic_bytes": nbytes, "achieved_gbs": round(nbytes / t / 1e9, 1)}
    epb = form.fes.kernel_info()
    out["elements_per_block"] = {"residual": epb[0], "tangent_fp64": epb[1], "tangent_fp32": epb[2]}
    if form.mixed:  # the FP32 tangent kernel the timed choice kept (1 coloured element kernel, 2 row kernel)
        out["tangent_fp32_kernel"] = form.asm.tangent_kernel()
    return out


def finish(args, p, world, t_mixed, t_e2e, t_plain, plain_info, infos, launches, mixed, n_nodes, spmv_ms, spmv_n,
           clocks, rel_diff, prof_solves, assembly=None):

    # roofline of the dominant kernel: the fused CG SpMV (two-kernel CG) or, when the tuner picked the persistent
    # CG, one CG iteration of it (SpMV streams plus the block-Jacobi inverse of the update phase)
    bpl, nb = spmv_bytes(mixed.asm, n_nodes, 4)
    kind, keep, _ = mixed.ls.kernel_info()
    persistent = kind >= 5
    if persistent:
        bpl += 9 * n_nodes * 4
    kname = ("pcg_persistent_kernel<float> (per CG iteration)" if persistent else
             "pcg_spmv_staged_kernel<float>" if kind > 0 else "pcg_spmv_kernel<float>")
    # per launch: a persistent launch is one CG solve (spmv_n counts its iterations), a staged launch one SpMV
    n_launch = max(prof_solves, 1) if persistent else max(spmv_n, 1)
    iters_per_launch = spmv_n / n_launch
    avg_s = spmv_ms / n_launch / 1e3
    bytes_per_launch = bpl * iters_per_launch
    pk = peaks()
    peak = pk["hbm_gbs"] if pk else 6800.0
    achieved = bytes_per_launch / avg_s / 1e9 if avg_s > 0 else None
    traffic = None
    tf = os.path.join(ROOT, "profiles", "cg_dram_traffic.json")
    if os.path.exists(tf) and not args.small:
        try:
            caps = json.load(open(tf))
            for t in (caps if isinstance(caps, list) else [caps]):
                if t.get("cg_kernel_kind") == kind and abs(t.get("l2_keep_fraction", -1) - keep) < 1e-9:
                    # DRAM bytes per CG iteration of that kernel and L2 keep share, from one ncu capture
                    traffic = round(t["dram_bytes_per_iteration"] * iters_per_launch)
        except (OSError, ValueError, KeyError, TypeError):
            traffic = None

    info0 = infos[-1]
    newton = [s.iterations for s in info0.solverInfos]
    out = {
        "metric": METRIC,
        "value": round(t_mixed, 4),
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_mixed * 1e3, 2),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 tangent/CG + fp64 residual (mixed); fp64 (plain)",
        "data": "synthetic (seeded jittered mesh, the configuration's shapes; no dataset involved)",
        "config": {"workload": p.name, "elements": p.mesh.n_elems, "nodes": n_nodes, "dofs": p.n_dofs,
                   "load_steps": p.load_steps, "tolerance": "||R||/||R0|| < 1e-8 every load step",
                   "material": "NeoHooke E=1000 nu=0.3", "parallelism": f"replicas x{world}",
                   "mixed_form": "FP32 tangent + FP32 block-Jacobi PCG (Eisenstat-Walker forcing), FP64 residual and "
                                 "Newton test" + (", Newton predictor = previous increment (the learned predictor's "
                                 "fallback; no trained model exists for this single load case)" if args.predictor
                                 else ", no Newton predictor"),
                   "plain_form": "FP64 tangent + FP64 block-Jacobi PCG to 1e-10, FP64 residual, no predictor",
                   "l2": "256 MB buffer written between timed load paths; working set > L2"},
        "plain_fp64": None if t_plain is None else
        {"s_per_load_path": round(t_plain, 4), "newton_iterations": plain_info.totalIterations,
         "cg_iterations": plain_info.totalLinearIterations},
        "mixed": {"newton_iterations": info0.totalIterations, "cg_iterations": info0.totalLinearIterations,
                  "newton_per_step": newton, "max_rel_diff_vs_plain": rel_diff,
                  "newton_iterations_as_cuda_graphs": mixed.nr.graph_iterations(),
                  "fp32_tangent_kernel": {1: "coloured element kernel", 2: "row kernel",
                                          3: "element blocks + gather"}.get(mixed.asm.tangent_kernel())},
        "speedup_vs_plain_fp64": None if t_plain is None else round(t_plain / t_mixed, 3),
        "e2e": {"value": round(t_e2e, 4), "unit": "s", "h2d_bytes_per_step": 8 * p.n_dofs,
                "d2h_bytes_per_step": 8 * p.n_dofs},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1) if achieved
                     else None, "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "traffic": traffic, "algorithmic_bytes_per_launch": round(bytes_per_launch),
                     "avg_launch_us": round(avg_s * 1e6, 3), "launches": n_launch,
                     "cg_iterations_per_launch": round(iters_per_launch, 2), "algorithmic_bytes_per_cg_iteration": bpl,
                     "us_per_cg_iteration": round(spmv_ms * 1e3 / max(spmv_n, 1), 3),
                     "cg_kernel_kind": kind, "l2_keep_fraction": keep,
                     "traffic_source": "ncu capture of the same kernel kind and L2 keep share, separate run "
                                       "(profiles/cg_dram_traffic.json)" if traffic is not None else None,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if pk else "fallback"},
        "clocks": clocks.summary(),
    }
    if assembly:
        out["assembly"] = assembly
    return out


# ---------------------------------------------------------------------------------------------------------
def cpu_threads():
    """Host threads the CPU oracle's CG uses: every core this process may run on."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except (AttributeError, OSError):
        return max(1, os.cpu_count() or 1)


def cpu_sample(p, plain_newton, plain_cg):
    """Bounded CPU sample of the headline workload on its own mesh (128x32x32, same seed): the oracle's residual and
    tangent assembly (serial, with the reference's per-(i,j) moduli evaluation) once and 300 iterations of its
    Jacobi-preconditioned CG (all host threads), scaled to the plain FP64 GPU run's Newton iterations and CG
    iterations.  That run's CG is block-Jacobi preconditioned; the oracle's point-Jacobi CG typically needs more
    iterations, so the estimate is a lower bound of the oracle's time."""
    import numpy as np

    import oracle

    oracle.set_threads(cpu_threads())
    o = oracle.from_problem(p, faithful=True)
    u = np.zeros(p.n_dofs)
    t0 = time.perf_counter()
    R = o.assemble_vector(u, 1.0 / p.load_steps)
    t1 = time.perf_counter()
    cp, ri, v, n = o.assemble_matrix_csc(u, 1.0 / p.load_steps)
    t2 = time.perf_counter()
    _, its, _ = oracle.cg_jacobi(cp, ri, v, -R, 0.0, 300)
    t3 = time.perf_counter()
    t_res, t_mat, t_it = t1 - t0, t2 - t1, (t3 - t2) / max(its, 1)
    est = plain_newton * (t_res + t_mat) + plain_cg * t_it
    return est, dict(t_residual_s=t_res, t_tangent_s=t_mat, t_cg_iteration_s=t_it)


def run_reference(args, world):
    """The reference's CPU implementation of the path (the oracle port; the reference itself cannot be built here)
    on the headline workload: complete load steps of the 128x32x32 jittered cantilever (same seed), each with the
    oracle's own Newton-Raphson to ||R||/||R0|| < 1e-8 and its Jacobi-preconditioned CG to 1e-10 (the reference's
    si_ConjugateGradient = Eigen's ConjugateGradient<Lower|Upper>, multithreaded over all host cores) on the
    serially assembled tangent (the reference's per-(i,j) moduli evaluation).  Load steps run in order from the
    undeformed state while they fit the time budget (at least one); the value is load_steps x the mean measured
    load-step time.  Warm-up: one residual assembly per warm-up step."""
    import numpy as np

    import oracle
    from ikarus_gb300 import problems

    p = problems.config2(load_steps=args.load_steps)
    T = cpu_threads()
    oracle.set_threads(T)
    o = oracle.from_problem(p, faithful=True)
    u = np.zeros(p.n_dofs)
    for _ in range(args.warmup):
        o.assemble_vector(u, 0.0)
    lam, dl = 0.0, 1.0 / p.load_steps
    steps, t_start = [], time.perf_counter()
    while len(steps) < min(args.steps, p.load_steps):
        t0 = time.perf_counter()
        u, lam, st = o.load_step(u, lam, dl, tol=1e-8, tol_mode=1, max_iter=30, solver=oracle.SOLVER_CG_JACOBI,
                                 cg_rtol=1e-10)
        st["s"] = time.perf_counter() - t0
        steps.append(st)
        log(f"reference load step {len(steps)}: {st['s']:.1f} s, newton {st['newton']:.0f}, cg {st['cg']:.0f}")
        if time.perf_counter() - t_start > args.ref_budget:
            break
    per_step = sum(s["s"] for s in steps) / len(steps)
    val = p.load_steps * per_step
    sample = (f"oracle port on the 128x32x32 jittered cantilever (same mesh and seed): load steps 1..{len(steps)} of "
              f"{p.load_steps} solved completely and timed (its own Newton to ||R||/||R0||<1e-8 and Jacobi-CG to "
              f"1e-10 on {T} threads; serial assembly with the reference's per-(i,j) moduli); value = "
              f"{p.load_steps} x the mean measured load-step time")
    detail = {"load_steps_measured": len(steps), "threads": T,
              "per_step": [{k: (float(f"{v:.4g}") if isinstance(v, float) else v) for k, v in s.items()}
                           for s in steps]}
    print(json.dumps({"metric": METRIC, "value": round(val, 2), "unit": "s", "impl": "reference", "n_gpus": world,
                      "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
                      "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
                      "config": {"workload": "cantilever_128x32x32_jittered", "elements": p.mesh.n_elems,
                                 "nodes": p.mesh.n_nodes, "dofs": p.n_dofs, "load_steps": p.load_steps,
                                 "tolerance": "||R||/||R0|| < 1e-8 every load step",
                                 "material": "NeoHooke E=1000 nu=0.3", "parallelism": f"replicas x{world}",
                                 "reference_form": "the reference's algorithm restated on the CPU (oracle): FP64 "
                                                   "assembly, Jacobi-preconditioned CG, Newton-Raphson under "
                                                   "LoadControl"},
                      "cpu_baseline": {"value": round(val, 2), "unit": "s", "cores": T, "kind": "port",
                                       "sample": sample, **detail},
                      "e2e": {"value": round(val, 2), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def run_spmv_only(args):
    """Tangent of the 128x32x32 cantilever at the undeformed state (FP32) and a fixed number of CG iterations on
    its external-load right-hand side, once per SpMV kernel choice in --spmv-kinds ("kind:keep" items, -1 =
    tuned): the workload of the SpMV ncu captures and of the kernel comparison."""
    import numpy as np

    import ikarus_gb300 as ikr
    from ikarus_gb300 import problems

    p = problems.config2(load_steps=20)
    fes, asm = problems.build_gpu(p, precision=args.spmv_precision)
    req = ikr.FERequirements(fes, None, 0.05)
    asm.matrix(req, dbc=ikr.DBCOption.Full, export=False)
    b = -asm.vector(req, dbc=ikr.DBCOption.Full)
    bpl, nb = spmv_bytes(asm, p.mesh.n_nodes, 4 if args.spmv_precision == 1 else 8)
    out = {"n_blocks": nb, "dofs": p.n_dofs, "graphs": not args.no_graphs, "spmv_bytes": bpl, "runs": []}
    for item in args.spmv_kinds.split(","):
        kind, _, keep = item.partition(":")
        ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=1e-30, max_iter=args.spmv_only)
        ls.set_launch(use_graphs=not args.no_graphs)
        ls.set_kernel(int(kind), float(keep) if keep else (0.0 if int(kind) >= 0 else -1.0))
        ls.compute(asm)
        k_used, keep_used, tuned_us = ls.kernel_info()
        rec = {"kind": k_used, "keep": keep_used, "tuned_us_per_iteration": round(tuned_us, 3)}
        for profiled in (False, True):
            ls.profile(profiled)
            t0 = time.perf_counter()
            try:
                ls.solve(asm, b)
            except ikr.IkarusError as e:  # the iteration limit is the point of this mode
                if e.code != -5 and "NOT_CONVERGED" not in str(e):
                    log(f"solve: {e}")
            wall = time.perf_counter() - t0
            it, rel = ls.last_info()
            rec["plain_us_per_iteration" if not profiled else "profiled_us_per_iteration"] = round(
                wall / max(it, 1) * 1e6, 2)
            if profiled:
                ms, n = ls.profile_read()
                rec["spmv_us"] = round(ms / max(n, 1) * 1e3, 3)
                rec["spmv_gbs"] = round(bpl / (ms / max(n, 1) / 1e3) / 1e9, 1) if ms > 0 else None
                rec["iterations"] = it
        if k_used >= 5:  # persistent kinds: the same iterations for two right-hand sides in one launch
            ls.profile(True)
            try:
                ls.solve(asm, np.stack([b, 0.5 * b + 1e-3], axis=1))
            except ikr.IkarusError as e:
                if e.code != -5 and "NOT_CONVERGED" not in str(e):
                    log(f"solve2: {e}")
            ms, n = ls.profile_read()
            rec["two_rhs_us_per_iteration"] = round(ms / max(n, 1) * 1e3, 3)
        ls.profile(False)
        out["runs"].append(rec)
        log(f"spmv-only: {rec}")
        del ls
    print(json.dumps(out))
    return 0


def run_batched(args):
    """512 independent cantilevers (random grids, lengths, materials, tip tractions), 10 load steps, every
    instance to ||R||/||R0|| < 1e-8 on every step: mixed form (FP32 tangent, batched FP32 CG, FP64 residual), alone
    and with precision escalation of the instances it takes out to FP64 (with its inexact-Newton controls, and with
    the plain form's settings), against the plain FP64 form of the same batched method (FP64 tangent and CG to
    1e-10).  The value is the escalated form's time."""
    import numpy as np
    import torch

    import ikarus_gb300 as ikr
    from ikarus_gb300 import problems

    bp = problems.batched_cantilevers(512, seed=7, load_steps=10)
    out = {"metric": "time to ||R||/||R0||<1e-8 on every load step for all 512 instances", "unit": "s",
           "higher_is_better": False, "config": {"workload": bp.name, "elements": bp.mesh.n_elems,
                                                  "dofs": bp.n_dofs, "instances": 512, "load_steps": 10,
                                                  "newton_backtracks": args.batched_backtracks,
                                                  "mixed_eta_max": args.batched_eta_max}}
    finals, status = {}, {}

    def settings(mixed):
        return ikr.NRSettings(tol=1e-8, maxIter=40, relative=True, eisenstat_walker=mixed,
                              linear_rtol=args.batched_eta_max if mixed else 1e-10, linear_rtol_min=1e-6,
                              linear_max_iter=20000, backtracks=args.batched_backtracks)

    def run_form(key, mixed, escalate=False):
        fes, asm = problems.build_gpu_batched(bp, precision=1 if mixed else 0)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(settings(mixed),
                                                            ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
        lc = ikr.LoadControl(nr, bp.load_steps)
        req, req0 = ikr.FERequirements(fes), ikr.FERequirements(fes)
        esc = None
        if escalate:
            # precision escalation: an instance the FP32 solver takes out in a step (inverted elements, no
            # convergence in maxIter, or a CG that cannot reach its tolerance in FP32) is solved again from the
            # step's start in FP64 and stays in FP64
            nr.set_batched_take_out(True)
            fes64, asm64 = problems.build_gpu_batched(bp, precision=0)
            # "ew": FP64 with the mixed form's inexact-Newton controls; "plain": the plain FP64 form's settings, so
            # that an escalated instance is solved from the step's start exactly as the plain form solves it
            nr64 = ikr.NewtonRaphson(asm64, ikr.NewtonRaphsonConfig(
                settings(escalate == "ew"), ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched)))
            req64 = ikr.FERequirements(fes64)
            lc.set_escalation(nr64, req64)
            esc = (fes64, asm64, nr64, req64)
        stream, ev0, ev1 = make_events(torch, fes.stream())
        times = []
        trace = []
        if args.batched_trace:
            # per batch Newton iteration: wall time (the batched Newton synchronises every iteration) and the largest
            # per-instance CG count, from the solver's observers
            t_state = {"t": 0.0, "lin": None}

            def on_nr(msg, s_):
                if msg == ikr.NonLinearSolverMessages.INIT:
                    t_state["t"] = time.perf_counter()
                    t_state["lin"] = np.zeros(len(bp.parts), dtype=np.int64)
                elif msg == ikr.NonLinearSolverMessages.ITERATION_ENDED:
                    now = time.perf_counter()
                    lin = nr.instance_linear_iterations()
                    d = lin - t_state["lin"]
                    t_state["lin"] = lin
                    trace.append((now - t_state["t"], int(d.max()), int((d > 0).sum())))
                    t_state["t"] = now
            nr.subscribe(on_nr)
        for k in range(args.warmup + args.steps):
            trace.clear()
            req.assign(req0)
            torch.cuda.synchronize()
            ev0.record(stream)
            info = lc.run(req)
            ev1.record(stream)
            ev1.synchronize()
            torch.cuda.synchronize()
            if k >= args.warmup:
                times.append(ev0.elapsed_time(ev1) / 1e3)
            log(f"batched {key}: {times[-1] if times else ev0.elapsed_time(ev1) / 1e3:.3f} s"
                f" success {info.success} newton {info.totalIterations} cg {info.totalLinearIterations}")
        its, rn, conv = nr.instance_info()
        conv = conv.copy()
        rec = {"s": round(sum(times) / len(times), 4), "success": bool(info.success),
               "newton_iterations_batch": info.totalIterations, "cg_iterations_sum": info.totalLinearIterations,
               "batched_cg_launches_per_run": nr.batched_cg_launches() // (args.warmup + args.steps)}
        if esc:
            escalated = lc.escalated()
            rec["escalated_to_fp64"] = int(escalated.sum())
            rec["escalated"] = [int(i) for i in np.nonzero(escalated)[0]]
            rec["escalated_after"] = {"element_inversion": int((escalated & (conv == -1)).sum()),
                                      "no_convergence_in_maxIter": int((escalated & (conv == -2)).sum()),
                                      "cg_unsolved_in_fp32": int((escalated & (conv == -4)).sum())}
            conv = lc.instance_status()
        rec.update({"instances_converged_last_step": int((conv == 1).sum()),
                    "instances_taken_out_element_inversion": int((conv == -1).sum()),
                    "instances_taken_out_not_converged": int((conv == -2).sum()),
                    "instances_taken_out_cg_unsolved": int((conv == -4).sum()),
                    "taken_out": [int(i) for i in np.nonzero(conv != 1)[0]]})
        if args.batched_trace and trace:
            tr = np.array(trace, dtype=float)
            capped = tr[:, 1] >= 0.95 * 20000
            order = np.argsort(-tr[:, 0])[:5]
            rec["trace"] = {
                "newton_iterations": len(tr), "wall_s": round(float(tr[:, 0].sum()), 3),
                "iterations_with_a_cg_at_its_cap": int(capped.sum()),
                "wall_s_in_those": round(float(tr[capped, 0].sum()), 3),
                "us_per_cg_iteration_in_those": round(float(tr[capped, 0].sum() / max(tr[capped, 1].sum(), 1)) * 1e6, 2),
                "slowest_iterations": [{"s": round(float(tr[k, 0]), 4), "largest_cg": int(tr[k, 1]),
                                        "instances_in_cg": int(tr[k, 2])} for k in order]}
        out[key] = rec
        finals[key], status[key] = req.globalSolution(), conv
        del lc, nr, asm, fes, esc

    run_form("mixed", True)
    run_form("plain_fp64", False)
    if not args.batched_trace:
        run_form("mixed_escalated", True, escalate="ew")
        run_form("mixed_escalated_to_plain", True, escalate="plain")

    def compare(a, b):
        both = np.nonzero((status[a] == 1) & (status[b] == 1))[0]
        diffs = []
        for i in both:
            sl = slice(3 * bp.node_offsets[i], 3 * bp.node_offsets[i + 1])
            ref = finals[b][sl]
            diffs.append(float(np.abs(finals[a][sl] - ref).max() / max(np.abs(ref).max(), 1e-300)))
        diffs = np.array(diffs)
        # both stop at ||R|| <= 1e-8 ||R0||, which leaves displacement differences up to ~cond(K) 1e-8; a difference
        # above 1e-3 of the displacement is another equilibrium (several exist for the beams loaded far beyond
        # their length)
        return {"same_instances_solved": bool(np.array_equal(status[a] == 1, status[b] == 1)),
                "instances_solved_by_both": int(len(both)),
                "solved_by_plain_only": [int(i) for i in np.nonzero((status[b] == 1) & (status[a] != 1))[0]],
                "solved_by_this_form_only": [int(i) for i in np.nonzero((status[a] == 1) & (status[b] != 1))[0]],
                "max_rel_diff_vs_plain": float(diffs.max()) if len(diffs) else None,
                "instances_on_another_branch": [int(both[k]) for k in np.nonzero(diffs > 1e-3)[0]],
                "max_rel_diff_vs_plain_same_branch": float(diffs[diffs <= 1e-3].max()) if (diffs <= 1e-3).any()
                else None}

    out["mixed_vs_plain"] = compare("mixed", "plain_fp64")
    if args.batched_trace:
        out["speedup_mixed_alone_vs_plain_fp64"] = round(out["plain_fp64"]["s"] / out["mixed"]["s"], 3)
        print(json.dumps(out))
        return
    out["mixed_escalated_vs_plain"] = compare("mixed_escalated", "plain_fp64")
    out["mixed_escalated_to_plain_vs_plain"] = compare("mixed_escalated_to_plain", "plain_fp64")
    out["speedup_escalated_to_plain_vs_plain_fp64"] = round(out["plain_fp64"]["s"] / out["mixed_escalated_to_plain"]["s"], 3)
    out["value"] = out["mixed_escalated"]["s"]
    out["speedup_vs_plain_fp64"] = round(out["plain_fp64"]["s"] / out["mixed_escalated"]["s"], 3)
    out["speedup_mixed_alone_vs_plain_fp64"] = round(out["plain_fp64"]["s"] / out["mixed"]["s"], 3)
    out["instances_per_s"] = round(512 / out["mixed_escalated"]["s"], 2)
    print(json.dumps(out))


def run_learned(args):
    """Learned Newton predictor on the 64x16x16 cantilever: load paths with random top pressure
    p(x) = sum a_k sin(k pi x / L) and tip traction; trained on --train-paths paths solved by the method without
    predictor, evaluated on --eval-paths held-out paths (Newton iterations and time to ||R||/||R0|| < 1e-8 on
    every step) against no predictor and against the previous-increment extrapolation."""
    import numpy as np
    import torch

    import ikarus_gb300 as ikr
    from ikarus_gb300 import problems

    p = problems.learned_cantilever(64, 16, 16, load_steps=20)
    fes, asm = problems.build_gpu(p, precision=1)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-5, linear_max_iter=200000)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver()))
    lc = ikr.LoadControl(nr, p.load_steps)
    req = ikr.FERequirements(fes)
    stream, ev0, ev1 = make_events(torch, fes.stream())
    pred = ikr.LearnedPredictor(fes, n_params=9, n_modes=64, width=256, depth=4,
                                capacity=args.train_paths * p.load_steps, seed=1)
    rng = np.random.default_rng(2025)

    def run(theta, kind, record=False):
        fes.clear_neumann()
        fes.add_neumann(*problems.learned_loads(p, theta))
        req.insertGlobalSolution(np.zeros(p.n_dofs))
        req.insertParameter(0.0)
        lc.set_predictor(kind, pred if (kind == 2 or record) else None, theta, record)
        torch.cuda.synchronize()
        ev0.record(stream)
        info = lc.run(req)
        ev1.record(stream)
        ev1.synchronize()
        return info, ev0.elapsed_time(ev1) / 1e3, lc.predictor_stats()

    t0 = time.perf_counter()
    for i in range(args.train_paths):
        info, _, _ = run(problems.sample_load_parameters(rng), 0, record=True)
        if not info.success:
            log(f"training path {i} did not converge")
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss, energy = pred.fit(epochs=300, batch=128, lr=1e-3)
    t_fit = time.perf_counter() - t0
    log(f"training data {t_data:.1f} s, fit {t_fit:.1f} s, loss {loss:.3e}, POD energy {energy:.6f}")
    res = {k: {"newton": 0, "cg": 0, "s": 0.0, "failed": 0} for k in ("none", "previous_increment", "learned")}
    kept = [0, 0]
    for j in range(args.eval_paths):
        theta = problems.sample_load_parameters(rng)
        for kind, name in ((0, "none"), (1, "previous_increment"), (2, "learned")):
            info, t, (acc, rej) = run(theta, kind)
            r = res[name]
            r["newton"] += info.totalIterations
            r["cg"] += info.totalLinearIterations
            r["s"] += t
            r["failed"] += 0 if info.success else 1
            if kind == 2:
                kept[0] += acc
                kept[1] += rej
    for r in res.values():
        r["s"] = round(r["s"] / args.eval_paths, 4)
    out = {"metric": "Newton iterations and time per held-out load path to ||R||/||R0||<1e-8 (learned predictor)",
           "config": {"workload": p.name, "dofs": p.n_dofs, "load_steps": p.load_steps, "train_paths":
                      args.train_paths, "eval_paths": args.eval_paths, "pod_modes": 64, "mlp": "4 x 256 GELU, BF16 "
                      "weights, FP32 accumulation"},
           "training": {"data_s": round(t_data, 2), "fit_s": round(t_fit, 2), "loss": loss, "pod_energy": energy},
           "results": res, "learned_predictions_kept": kept[0], "learned_predictions_rejected": kept[1],
           "newton_saving_vs_none": round(1 - res["learned"]["newton"] / max(1, res["none"]["newton"]), 4),
           "time_saving_vs_none": round(1 - res["learned"]["s"] / max(1e-9, res["none"]["s"]), 4)}
    print(json.dumps(out))


def run_eas(args):
    """Nearly incompressible EAS block (64x64x16, 9-parameter GL EAS, nu = 0.4999, pressure 0 -> 50 on the centred
    top patch, 25 load steps), every step to ||R||/||R0|| < 1e-8: plain FP64 form against the mixed form (FP32
    global tangent and block-Jacobi CG as the preconditioner of an FP64 outer flexible GMRES on the FP64 twin of
    the tangent, FP64 EAS condensation and residual), with the per-step error of the mixed displacements against
    the plain ones."""
    import numpy as np
    import torch

    import ikarus_gb300 as ikr
    from ikarus_gb300 import problems

    nx, ny, nz = (int(v) for v in args.eas_size.split(","))
    p = problems.eas_block(nx, ny, nz, load_steps=args.eas_steps)
    out = {"metric": "time to ||R||/||R0||<1e-8 on every load step (nearly incompressible EAS block)", "unit": "s",
           "higher_is_better": False,
           "config": {"workload": p.name, "elements": p.mesh.n_elems, "dofs": p.n_dofs, "load_steps": p.load_steps,
                      "steps_run": args.eas_first_steps if 0 < args.eas_first_steps < p.load_steps else p.load_steps,
                      "eas": "GreenLagrange E9", "nu": 0.4999, "predictor": args.eas_predictor,
                      "newton_backtracks": args.backtracks, "mixed_cg_cap": args.eas_cg_cap,
                      "mixed_outer": {"restart": args.eas_restart, "inner_rtol": args.eas_inner_rtol,
                                      "inner_max_iter": args.eas_cg_cap}}}
    per_step = {}
    for mixed in (False, True):
        fes, asm = problems.build_gpu(p, precision=1 if mixed else 0)
        if mixed:
            st = ikr.NRSettings(tol=1e-8, maxIter=80, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                                linear_rtol_min=1e-5, linear_max_iter=args.eas_cg_cap,
                                backtracks=args.backtracks)
        else:
            st = ikr.NRSettings(tol=1e-8, maxIter=40, relative=True, linear_rtol=1e-10, linear_max_iter=1000000,
                                backtracks=args.backtracks)
        ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi)
        if mixed and args.eas_restart > 0:
            ls.set_fp64_outer(restart=args.eas_restart, inner_rtol=args.eas_inner_rtol,
                              inner_max_iter=args.eas_cg_cap)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ls))
        k = args.eas_first_steps if 0 < args.eas_first_steps < p.load_steps else p.load_steps
        lc = ikr.LoadControl(nr, k, (0.0, k / p.load_steps))
        if args.eas_predictor:
            lc.set_predictor(1)
        req = ikr.FERequirements(fes)
        us = []

        def obs(msg, state, req=req, us=us):
            if msg == ikr.ControlMessages.STEP_ENDED:
                us.append(req.globalSolution())

        lc.subscribe(obs)
        stream, ev0, ev1 = make_events(torch, fes.stream())
        torch.cuda.synchronize()
        ev0.record(stream)
        key = "mixed" if mixed else "plain_fp64"
        try:
            info = lc.run(req)
        except ikr.IkarusError as e:  # e.g. an iterate that inverts an element (the reference aborts there)
            ev1.record(stream)
            ev1.synchronize()
            out[key] = {"s": round(ev0.elapsed_time(ev1) / 1e3, 3), "success": False, "error": str(e),
                        "steps_completed": max(len(us) - 1, 0), "spmv_kernel": ls.kernel_info()[:2]}
            per_step[key] = us
            log(f"eas {key}: failed after {out[key]['s']} s: {e}")
            del lc, nr, ls, asm, fes
            continue
        ev1.record(stream)
        ev1.synchronize()
        t = ev0.elapsed_time(ev1) / 1e3  # includes the observer's per-step downloads
        out[key] = {"s": round(t, 3), "success": bool(info.success), "newton_iterations": info.totalIterations,
                    "cg_iterations": info.totalLinearIterations,
                    "newton_per_step": [si.iterations for si in info.solverInfos], "spmv_kernel": ls.kernel_info()[:2]}
        per_step[key] = us
        log(f"eas {key}: {t:.2f} s success {info.success} newton {info.totalIterations} "
            f"cg {info.totalLinearIterations}")
        del lc, nr, ls, asm, fes
    if len(per_step["mixed"]) == len(per_step["plain_fp64"]):
        out["mixed"]["max_rel_diff_vs_plain_per_step"] = [
            float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
            for a, b in zip(per_step["mixed"], per_step["plain_fp64"])]
    out["value"] = out["mixed"]["s"] if out["mixed"]["success"] else None
    if out["mixed"]["success"] and out["plain_fp64"]["success"]:
        out["speedup_vs_plain_fp64"] = round(out["plain_fp64"]["s"] / out["mixed"]["s"], 3)
    print(json.dumps(out))


def run_path_following(args):
    """Arc-length path following (PathFollowing + NewtonRaphsonWithSubsidiaryFunction) on the 128x32x32 cantilever:
    `steps` arc-length steps sized so that the first step takes Dlambda = 1 / steps (s = sqrt(2) psi / steps with
    psi = ||K^-1 Fext|| from a one-step calibration run of the plain form), every solve to
    sqrt(||R||^2 + f^2) <= 1e-8 x its initial value.  Each Newton iteration is two CG solves with the same tangent
    (K dR = -R, K dL = Fext0).  Plain FP64 form against the mixed form; the CPU figure is the oracle port's
    per-element / per-nonzero costs scaled to the plain run's Newton and CG counts."""
    import numpy as np
    import torch

    import ikarus_gb300 as ikr
    from ikarus_gb300 import problems

    steps = args.path_following
    p = problems.config2(load_steps=steps)
    out = {"metric": f"time per arc-length path ({steps} steps, sqrt(||R||^2+f^2) <= 1e-8 x initial, every step)",
           "unit": "s", "higher_is_better": False,
           "config": {"workload": "cantilever_128x32x32_jittered", "elements": p.mesh.n_elems, "dofs": p.n_dofs,
                      "path_following": "ArcLength, AdaptiveStepSizing::NoOp", "steps": steps,
                      "bordered_solve": "two CG columns one after the other" if args.no_multi_rhs else
                                        "two CG columns in one persistent launch (one matrix stream per iteration)",
                      "load_column": "from zero" if args.no_warm_start else
                                     "warm start from the previous Newton iteration's solution",
                      "material": "NeoHooke E=1000 nu=0.3", "l2": "256 MB buffer written before each timed path"}}
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    s_hat = None
    finals = {}
    for mixed in ((True,) if args.pf_mixed_only else (False, True)):
        fes, asm = problems.build_gpu(p, precision=1 if mixed else 0)
        ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi)
        ls.set_multi_rhs(not args.no_multi_rhs)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(solver_settings(ikr, mixed, (args.eta_max, args.eta_min)),
                                                            ls))
        req = ikr.FERequirements(fes)
        stream, ev0, ev1 = make_events(torch, fes.stream())
        if s_hat is None:  # calibration: psi = ||DD0|| of the initial prediction (plain form)
            cal = ikr.PathFollowing(nr, 1, 1.0, ikr.ArcLength())
            assert cal.run(req).success
            s_hat = np.sqrt(2.0) * cal.subsidiary_args()["psi"] / steps
            out["config"]["arc_length"] = s_hat
            del cal
        pf = ikr.PathFollowing(nr, steps, s_hat, ikr.ArcLength())
        pf.set_warm_start(not args.no_warm_start)
        times = []
        for k in range(args.warmup + args.steps):
            req.insertGlobalSolution(np.zeros(p.n_dofs))
            req.insertParameter(0.0)
            flush.zero_()
            torch.cuda.synchronize()
            ev0.record(stream)
            info = pf.run(req)
            ev1.record(stream)
            ev1.synchronize()
            assert info.success, "arc-length path failed"
            if k >= args.warmup:
                times.append(ev0.elapsed_time(ev1) / 1e3)
            log(f"path following {'mixed' if mixed else 'plain'}: {ev0.elapsed_time(ev1) / 1e3:.3f} s, newton "
                f"{info.totalIterations}, cg {info.totalLinearIterations}, lambda {req.parameter():.6f}, "
                f"{pf.stats()}")
        key = "mixed" if mixed else "plain_fp64"
        out[key] = {"s": round(sum(times) / len(times), 4), "newton_iterations": info.totalIterations,
                    "cg_iterations": info.totalLinearIterations,
                    "newton_per_step": [si.iterations for si in info.solverInfos],
                    "final_lambda": req.parameter(), "psi": pf.subsidiary_args()["psi"], **pf.stats(),
                    "spmv_kernel": ls.kernel_info()[:2]}
        finals[key] = req.globalSolution()
        del pf, nr, ls, req, asm, fes
    out["value"] = out["mixed"]["s"]
    if args.pf_mixed_only:
        print(json.dumps(out))
        return
    out["speedup_vs_plain_fp64"] = round(out["plain_fp64"]["s"] / out["mixed"]["s"], 2)
    out["mixed"]["rel_psi_diff_vs_plain"] = abs(out["mixed"]["psi"] / out["plain_fp64"]["psi"] - 1.0)
    out["mixed"]["max_rel_diff_vs_plain"] = float(np.abs(finals["mixed"] - finals["plain_fp64"]).max()
                                                  / np.abs(finals["plain_fp64"]).max())
    if not args.no_cpu_baseline:
        v, parts = cpu_sample(p, out["plain_fp64"]["newton_iterations"], out["plain_fp64"]["cg_iterations"])
        out["cpu_baseline"] = {"value": round(v, 2), "unit": "s", "cores": cpu_threads(), "kind": "port",
                               "sample": "oracle port on the 128x32x32 mesh itself: one residual + tangent assembly "
                                         "(serial) and 300 Jacobi-CG iterations (all host threads), scaled to the "
                                         "plain FP64 path's Newton / CG counts (a lower bound: see the headline "
                                         "line)", **{k: round(x, 6) for k, x in parts.items()}}
    print(json.dumps(out))


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, world)
        return
    if args.spmv_only:
        return run_spmv_only(args)
    if args.path_following:
        return run_path_following(args)
    if args.config == 3:
        return run_batched(args)
    if args.config == 4:
        return run_learned(args)
    if args.config == 5:
        return run_eas(args)
    if args.two_level_only:
        import torch

        import ikarus_gb300 as ikr
        from ikarus_gb300 import problems
        p = problems.config2(load_steps=args.load_steps)
        print(json.dumps({"two_level": run_two_level(args, ikr, torch, problems, p, None, None)}))
        return
    out, p = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline and not args.small and out["plain_fp64"]:
            v, parts = cpu_sample(p, out["plain_fp64"]["newton_iterations"], out["plain_fp64"]["cg_iterations"])
            out["cpu_baseline"] = {"value": round(v, 2), "unit": "s", "cores": cpu_threads(), "kind": "port",
                                   "sample": "oracle port on the 128x32x32 mesh itself: one residual + tangent "
                                             "assembly (serial, reference-faithful moduli) and 300 Jacobi-CG "
                                             "iterations (all host threads), scaled to this run's plain FP64 Newton "
                                             "and CG counts (block-Jacobi CG counts: a lower bound for the oracle's "
                                             "point-Jacobi CG); bench.py --impl reference times complete load steps",
                                   **{k: round(x, 6) for k, x in parts.items()}}
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
