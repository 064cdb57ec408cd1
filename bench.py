#!/usr/bin/env python3
"""DOF-stage updates/s of the P2DE.jl 2D Euler DG step (RHS + subcell limiter +
SSP-RK3) on GB300.

Workload (the large, limiter-heavy configuration): double Mach reflection on
[0,4]x[0,1], 480x120 quads, N=3 (16 GLL nodes per element, 921,600 nodes), FP64,
CFL 0.5, reflecting wall + inflow + outflow + moving-shock boundaries. A "step" is one
SSP-RK3 step (three right-hand sides and stage updates); a DOF-stage update is one
node (all four components) advanced through one RK stage.

  value : device-resident state, CUDA-graph replay of the step, CUDA events on the
          launching stream, K timed steps after W warm-up steps.
  e2e   : the same steps through the public C ABI with host buffers: every step copies
          Uq from pinned host memory to the device (p2de_set_Uq), steps
          (p2de_ssp33_step) and reads Uq back (p2de_get_field).
  roofline: stage kernel A (low-order RHS, high-order RHS, limiter bounds), FP64-pipe
          bound; achieved = algorithmic FP64 operations / its mean event-timed launch;
          peak = FP64 FMA throughput probed on this GPU in this run.
  cpu_baseline / --impl reference: the FP64 CPU restatement (oracle/) with OpenMP on
          all host cores; Julia, the reference's language, is not available.
Multi-GPU: independent replicas (the path has no exchange between solves).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from ctypes import byref, c_double, c_int64, c_uint64
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "p2de.jl_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "DOF-stage updates/s, 2D Euler N=3; served solves/s + p99 vs plain, same L1 err"
UNIT = "DOF-stage updates/s"

# stage kernel A on this workload from one ncu capture
# (profiles/k_stage_a_dmr480x120_n3_fp64.md): DRAM traffic per launch
# (dram__bytes_read.sum + dram__bytes_write.sum) and the FP64 pipe's busy fraction
KERNEL_A_TRAFFIC_BYTES = 147.9e6
KERNEL_A_FP64_PIPE_BUSY = 0.825


def fma_probe_library():
    """libp2de_probe.so (built beside the solver library by build()): the FP64/FP32 FMA
    throughput probe whose FP64 figure is kernel A's roofline denominator."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("p2de_build", ROOT / "p2de.jl_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    lib = ctypes.CDLL(str(mod.build_probe()))
    lib.p2de_probe_fma_peak.argtypes = [ctypes.c_int, ctypes.c_int32, ctypes.POINTER(c_double)]
    lib.p2de_probe_fma_peak.restype = ctypes.c_int
    return lib


def workload(name: str, precision: str, basis: str = "lobatto", mesh: str = ""):
    """The benchmark's workloads; mesh "KXxKY" replaces the double Mach reflection's 480x120
    (a smaller case for profiler captures)."""
    from p2de import problems
    from p2de.types import GaussCollocation, NodewiseScaledExtrapolation, PositivityBound, SubcellLimiter

    kx, ky = (480, 120) if not mesh else tuple(int(v) for v in mesh.lower().split("x"))

    if name == "dmr" and basis == "gauss":
        # the reference's Gauss configuration (examples/2D/kelvin-helmholtz.jl:44-55):
        # GaussCollocation, NodewiseScaledExtrapolation, SubcellLimiter(PositivityBound)
        param, ic, bcf = problems.double_mach_reflection(
            N=3, Kx=kx, Ky=ky, T=0.2, precision=precision, approximation_basis=GaussCollocation(),
            entropyproj_limiter=NodewiseScaledExtrapolation(), rhs_limiter=SubcellLimiter(bound=PositivityBound()))
        desc = (f"double Mach reflection {kx}x{ky} quads, N=3, SSP-RK3 CFL 0.5, GaussCollocation + "
                "NodewiseScaledExtrapolation, positivity bound")
    elif name == "dmr":
        param, ic, bcf = problems.double_mach_reflection(N=3, Kx=kx, Ky=ky, T=0.2, precision=precision)
        desc = f"double Mach reflection {kx}x{ky} quads, N=3, SSP-RK3 CFL 0.5"
    elif name == "kh256":
        param, ic, bcf = problems.kelvin_helmholtz(N=3, Kx=256, Ky=256, T=1.0, precision=precision)
        desc = "Kelvin-Helmholtz 256x256 quads, N=3, SSP-RK3 CFL 0.5"
    else:
        raise SystemExit(f"unknown workload {name}")
    return param, ic, bcf, desc


def build_descriptor(param, ic, bcf):
    import p2de
    from p2de import solver as S

    md = S.mesh_for(param)  # the nodes of param's basis; a Line mesh for 1D Euler
    bc = bcf(param, md)
    desc = S.make_descriptor(param, md, bc)
    U0 = S.evaluate_initial_condition(param, md, ic)
    return md, bc, desc, U0


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"),
                stderr=subprocess.DEVNULL,
            )
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        finally:
            if self.path:
                try:
                    os.unlink(self.path)
                except OSError:
                    pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(rows),
            "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None,
        }


def cpu_baseline(desc, U0, nodes: int, budget_s: float = 12.0) -> dict:
    """The FP64 oracle with OpenMP on every host core, over as many full steps of the
    workload as fit in `budget_s` (at least one)."""
    from oracle.binding import Oracle, num_threads

    cores = os.cpu_count() or 1
    o = Oracle(desc, nthreads=cores)
    o.set_Uq(U0)
    t = 0.0
    t0 = time.perf_counter()
    steps = 0
    while True:
        t, _ = o.step(t)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    o.close()
    return {
        "value": nodes * 3 * steps / el,
        "unit": UNIT,
        "cores": num_threads(),
        "kind": "port",
        "sample": f"{steps} full SSP-RK3 steps of the same workload from t=0 ({el:.1f} s, FP64 C++ restatement of P2DE.jl with OpenMP)",
    }


def run_reference(args):
    """--impl reference: the CPU restatement on all host cores, same workload/metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    param, ic, bcf, wdesc = workload(args.workload, "fp64", args.basis, args.mesh)
    md, bc, desc, U0 = build_descriptor(param, ic, bcf)
    from oracle.binding import Oracle, num_threads

    cores = os.cpu_count() or 1
    o = Oracle(desc, nthreads=cores)
    o.set_Uq(U0)
    nodes = desc.K * desc.Nq
    t = 0.0
    for _ in range(args.warmup):
        t, _ = o.step(t)
    budget = 150.0
    t0 = time.perf_counter()
    steps = 0
    while steps < args.steps:
        t, _ = o.step(t)
        steps += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = nodes * 3 * steps / el
    sample = f"{steps} of {args.steps} requested full SSP-RK3 steps (time-capped at {budget:.0f} s), FP64 C++ restatement of P2DE.jl, OpenMP"
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": wdesc, "elements": desc.K, "nodes": nodes},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": num_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _advance(solver, nsteps, t):
    """nsteps graph-replayed steps from time t; returns (t, steps done)."""
    tt, n = c_double(t), c_int64()
    solver._check(solver.lib.p2de_ssp33_advance(solver.handle, nsteps, byref(tt), byref(n)))
    return tt.value, n.value


def _timed_alone(param, md, desc, U0, warmup, steps, tune=True):
    """One solve alone on the single-solve path: (seconds for `steps` steps after
    `warmup`, final Uq, steps done). Device time by CUDA events on the solver's stream."""
    import torch

    from p2de import abi
    from p2de import solver as S

    g = S.Solver(param, md, desc)
    st = torch.cuda.Stream()
    g._check(g.lib.p2de_set_stream(g.handle, ctypes.c_void_p(st.cuda_stream)))
    g.set_Uq(U0)
    if tune:
        g.autotune()
    t, _ = _advance(g, warmup, 0.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    t, n = _advance(g, steps, t)
    e1.record(st)
    torch.cuda.synchronize()
    U = g.get_field(abi.FIELD_UQ)
    g.close()
    return e0.elapsed_time(e1) * 1e-3, U, n


def run_batch64(args):
    """Many uneven solves in one persistent launch per RK stage: 64 four-quadrant
    Riemann problems (meshes 32^2..192^2, N in {2,3,4}), mixed precision, autotuned
    elements-per-block, CUDA-graph-captured step; against each solve alone on the
    plain (FP64, single-solve) path. A step advances every member by one SSP-RK3 step."""
    import torch

    from p2de import workloads as W
    from p2de.batch import Batch, solve_bytes

    torch.cuda.set_device(0)
    cases = W.riemann_batch_cases(64, seed=3)
    steps, warm = args.steps, args.warmup
    built = {p: [W.build_case(c, p) for c in cases] for p in ("mixed", "mixed-acc64", "fp64")}
    nodes = np.array([c.nodes for c in cases], dtype=np.float64)
    out = {}
    finals = {}
    for prec in ("mixed", "mixed-acc64", "fp64"):
        descs = [b[3] for b in built[prec]]
        pool = int(sum(solve_bytes(d) for d in descs) * 1.05) + (64 << 20)
        b = Batch(pool_bytes=pool, max_solves=len(cases), precision=prec)
        slots = [b.add(bb[3], bb[4]) for bb in built[prec]]
        t0 = time.perf_counter()
        tuned = b.autotune() if not args.no_autotune else {}
        tune_s = time.perf_counter() - t0
        b.step(warm)
        s0 = b.states()[slots, 1].copy()
        with ClockSampler(0) as clk:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.step(steps)
            el = time.perf_counter() - t0
        s1 = b.states()[slots, 1]
        dof = float(np.sum(nodes * 3 * (s1 - s0)))
        out[prec] = {"value": dof / el, "seconds": el, "steps_per_member_min": int(np.min(s1 - s0)),
                     "autotuned_elements_per_block": {str(k): v for k, v in tuned.items()},
                     "autotune_s": tune_s, "pool_bytes": pool, "clocks": clk.summary()}
        finals[prec] = [b.Uq(s) for s in slots]
        b.close()
    # each member alone on the single-solve path, same warm-up and step count
    alone = {}
    ref_U = []
    for prec in ("fp64", "mixed"):
        tot, dof = 0.0, 0.0
        for c, (param, md, bc, desc, U0) in zip(cases, built[prec]):
            sec, U, n = _timed_alone(param, md, desc, U0, warm, steps, tune=not args.no_autotune)
            tot += sec
            dof += c.nodes * 3 * n
            if prec == "fp64":
                ref_U.append(U)
        alone[prec] = {"value": dof / tot, "seconds": tot}
    # accuracy of the batched mixed members against the FP64 solves (same steps)
    errs, errs64 = [], []
    for c, bb, U, U64, R in zip(cases, built["fp64"], finals["mixed"], finals["mixed-acc64"], ref_U):
        Wq = W.quadrature_weights(c.N, bb[1].geom)
        errs.append(W.relative_errors(U, R, Wq)["rho"]["L1"])
        errs64.append(W.relative_errors(U64, R, Wq)["rho"]["L1"])
    fp64_batch_vs_alone = max(float(np.max(np.abs(U - R))) for U, R in zip(finals["fp64"], ref_U))
    total_nodes = int(nodes.sum())
    line = {
        "metric": METRIC,
        "value": out["mixed"]["value"],
        "unit": UNIT,
        "n_gpus": 1,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": 1e3 * out["mixed"]["seconds"] / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64+f32 (mixed)",
        "data": "synthetic",
        "config": {
            "workload": "64 four-quadrant Riemann problems, meshes 32^2..192^2, N in {2,3,4}, one batch",
            "nodes": total_nodes,
            "timing": "host wall clock around the batched steps (synchronised); alone: CUDA events",
            "l2": "working set ~%.1f GB > L2" % (out["mixed"]["pool_bytes"] / 1e9),
        },
        "batched_mixed": out["mixed"],
        "batched_mixed_acc64": out["mixed-acc64"],
        "batched_fp64": out["fp64"],
        "alone_fp64_plain": alone["fp64"],
        "alone_mixed": alone["mixed"],
        "speedup_batched_mixed_vs_alone_fp64": out["mixed"]["value"] / alone["fp64"]["value"],
        "rho_L1_rel_err_mixed_vs_fp64": {"max": max(errs), "median": float(np.median(errs))},
        "rho_L1_rel_err_mixed_acc64_vs_fp64": {"max": max(errs64), "median": float(np.median(errs64))},
        "fp64_batched_vs_alone_max_abs_diff": fp64_batch_vs_alone,
    }
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Continuous batching: a Poisson stream of solves (Kelvin-Helmholtz, four-quadrant
    Riemann, isentropic vortex; meshes 16^2..256^2, N 2..5) submitted to the native
    server at their arrival times, against a one-at-a-time queue on the plain FP64
    single-solve path fed by the same stream. Latency = completion - arrival."""
    import threading

    import torch

    from p2de import abi
    from p2de import solver as S
    from p2de import workloads as W
    from p2de.batch import Server

    torch.cuda.set_device(0)
    rates = [float(r) for r in args.serve_rates.split(",")]
    lines = []
    for rate in rates:
        stream = W.serving_stream(args.serve_requests, rate, seed=5, time_scale=args.serve_time_scale)
        sp = args.serve_precision
        built = {p: [W.build_case(c, p) for c in stream] for p in (sp, "fp64")}
        # served (continuous batching)
        sv = Server(hbm_budget_bytes=int(args.serve_budget_gb * 1e9), max_active=args.serve_max_active,
                    steps_per_tick=args.serve_steps_per_tick, precision=sp)
        rids = [None] * len(stream)
        t_start = time.perf_counter()

        def feeder():
            for i, (c, bb) in enumerate(zip(stream, built[sp])):
                d = t_start + c.arrival - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                rids[i] = sv.submit(bb[3], bb[4])

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        served_U, lat = [], []
        for rid in rids:
            while sv.wait(rid, 600.0) < Server.DONE:
                pass
            info = sv.poll(rid)
            lat.append(info.latency_s)
            served_U.append(sv.result(rid))
        makespan = time.perf_counter() - t_start
        stats = sv.stats()
        sv.close()
        # one-at-a-time plain FP64 queue over the same stream
        plat, plain_U = [], []
        t_start = time.perf_counter()
        busy = 0.0
        for c, (param, md, bc, desc, U0) in zip(stream, built["fp64"]):
            now = time.perf_counter() - t_start
            if now < c.arrival:
                time.sleep(c.arrival - now)
            t1 = time.perf_counter()
            g = S.Solver(param, md, desc)
            g.set_Uq(U0)
            tt, n, dtl = c_double(), c_int64(), c_double()
            g._check(g.lib.p2de_ssp33(g.handle, byref(tt), byref(n), byref(dtl)))
            plain_U.append(g.get_field(abi.FIELD_UQ))
            g.close()
            t2 = time.perf_counter()
            busy += t2 - t1
            plat.append(t2 - t_start - c.arrival)
        plain_makespan = time.perf_counter() - t_start
        errs = []
        for c, bb, U, R in zip(stream, built["fp64"], served_U, plain_U):
            errs.append(W.relative_errors(U, R, W.quadrature_weights(c.N, bb[1].geom))["rho"]["L1"])
        lines.append({
            "rate_req_per_s": rate,
            "requests": len(stream),
            "served": {"solves_per_s": len(stream) / makespan, "p50_s": float(np.percentile(lat, 50)),
                       "p99_s": float(np.percentile(lat, 99)), "makespan_s": makespan, "ticks": stats["ticks"],
                       "busy_s": stats["busy_s"]},
            "plain_queue": {"solves_per_s": len(stream) / plain_makespan, "p50_s": float(np.percentile(plat, 50)),
                            "p99_s": float(np.percentile(plat, 99)), "makespan_s": plain_makespan, "busy_s": busy},
            "rho_L1_rel_err_served_vs_fp64": {"max": max(errs), "median": float(np.median(errs))},
        })
    line = {
        "metric": METRIC,
        "value": lines[-1]["served"]["solves_per_s"],
        "unit": "solves/s",
        "n_gpus": 1,
        "higher_is_better": True,
        "dtype": f"f64+f32 ({args.serve_precision})",
        "data": "synthetic",
        "config": {
            "workload": "Poisson stream of 2D Euler solves (KH, four-quadrant Riemann, isentropic vortex), "
                        "meshes 16^2..256^2, N 2..5",
            "t_final": f"U[0.05, 0.5] x {args.serve_time_scale}",
            "hbm_budget_gb": args.serve_budget_gb,
            "max_active": args.serve_max_active,
            "steps_per_tick": args.serve_steps_per_tick,
        },
        "sweep": lines,
    }
    print(json.dumps(line), flush=True)


def run_mixed_report(args):
    """Mixed precision against all-FP64 on Kelvin-Helmholtz 256^2 to T: L1/Linf per
    component, total-entropy drift, positivity margin, speedup."""
    import torch

    from p2de import abi, problems
    from p2de import solver as S
    from p2de import workloads as W

    torch.cuda.set_device(0)
    res = {}
    for N in [int(x) for x in args.mixed_N.split(",")]:
        runs = {}
        for prec in ("fp64", "mixed", "mixed-acc64"):
            param, ic, bcf = problems.kelvin_helmholtz(N=N, Kx=256, Ky=256, T=args.T, precision=prec)
            md, bc, desc, U0 = build_descriptor(param, ic, bcf)
            Wq = W.quadrature_weights(N, md.geom)
            g = S.Solver(param, md, desc)
            st = torch.cuda.Stream()
            g._check(g.lib.p2de_set_stream(g.handle, ctypes.c_void_p(st.cuda_stream)))
            g.set_Uq(U0)
            if not args.no_autotune:
                g.autotune()
            t, steps, dev_s = 0.0, 0, 0.0
            minr, mine = np.inf, np.inf
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            while t < args.T:
                e0.record(st)
                t, n = _advance(g, 200, t)
                e1.record(st)
                torch.cuda.synchronize()
                dev_s += e0.elapsed_time(e1) * 1e-3
                steps += n
                r, e = c_double(), c_double()
                g._check(g.lib.p2de_min_rho_rhoe(g.handle, byref(r), byref(e)))
                minr, mine = min(minr, r.value), min(mine, e.value)
                if n == 0:
                    break
            mins = np.zeros(6)
            g._check(g.lib.p2de_stage_minima(g.handle, abi.dptr(mins)))
            U = g.get_field(abi.FIELD_UQ)
            g.close()
            runs[prec] = {"U": U, "t": t, "steps": steps, "seconds": dev_s, "min_rho": minr, "min_rhoe": mine,
                          "entropy0": W.total_entropy(U0, Wq), "entropyT": W.total_entropy(U, Wq),
                          "nodes": desc.K * desc.Nq, "last_stage_minima": mins.tolist()}
        f, m, m64 = runs["fp64"], runs["mixed"], runs["mixed-acc64"]
        res[f"N={N}"] = {
            "T": args.T,
            "steps": {p: r["steps"] for p, r in runs.items()},
            "errors_mixed_vs_fp64": W.relative_errors(m["U"], f["U"], W.quadrature_weights(N, md.geom)),
            "errors_mixed_acc64_vs_fp64": W.relative_errors(m64["U"], f["U"], W.quadrature_weights(N, md.geom)),
            "entropy_drift_rel": {p: (r["entropyT"] - r["entropy0"]) / abs(r["entropy0"]) for p, r in runs.items()},
            "min_rho": {p: r["min_rho"] for p, r in runs.items()},
            "min_rhoe": {p: r["min_rhoe"] for p, r in runs.items()},
            "dof_stage_per_s": {p: r["nodes"] * 3 * r["steps"] / r["seconds"] for p, r in runs.items()},
            "speedup_mixed": (m["nodes"] * 3 * m["steps"] / m["seconds"]) / (f["nodes"] * 3 * f["steps"] / f["seconds"]),
            "speedup_mixed_acc64": (m64["nodes"] * 3 * m64["steps"] / m64["seconds"]) / (f["nodes"] * 3 * f["steps"] / f["seconds"]),
        }
    print(json.dumps({"metric": METRIC, "unit": UNIT, "workload": "Kelvin-Helmholtz 256x256, mixed vs FP64",
                      "data": "synthetic", "report": res}), flush=True)


def run_limiter_report(args):
    """The double Mach reflection 480x120 N=3 step (FP64) under every limiter the one-solve
    path has, in both bound semantics: DOF-stage updates/s and ms per step for each, same
    steps and warm-up, autotuned elements per block."""
    import torch

    from p2de import problems
    from p2de.types import (
        GaussCollocation,
        HennemannShockCapture,
        NodewiseScaledExtrapolation,
        PositivityAndCellEntropyBound,
        PositivityAndMinEntropyBound,
        PositivityAndRelaxedCellEntropyBound,
        PositivityAndRelaxedMinEntropyBound,
        PositivityBound,
        SubcellLimiter,
        TVDAndMinEntropyBound,
        TVDBound,
        ZhangShuLimiter,
    )

    torch.cuda.set_device(0)
    limiters = {
        "positivity-and-cell-entropy (bench default)": SubcellLimiter(bound=PositivityAndCellEntropyBound()),
        "positivity": SubcellLimiter(bound=PositivityBound()),
        "positivity + hennemann": SubcellLimiter(bound=PositivityBound(), shockcapture=HennemannShockCapture()),
        "tvd": SubcellLimiter(bound=TVDBound()),
        "min-entropy": SubcellLimiter(bound=PositivityAndMinEntropyBound()),
        "relaxed-min-entropy": SubcellLimiter(bound=PositivityAndRelaxedMinEntropyBound()),
        "tvd-and-min-entropy": SubcellLimiter(bound=TVDAndMinEntropyBound()),
        "relaxed-cell-entropy(0.5)": SubcellLimiter(bound=PositivityAndRelaxedCellEntropyBound(beta=0.5)),
        "zhang-shu": ZhangShuLimiter(),
        "gauss + scaled extrapolation, positivity": SubcellLimiter(bound=PositivityBound()),
        "gauss + scaled extrapolation, zhang-shu": ZhangShuLimiter(),
    }
    gauss = dict(approximation_basis=GaussCollocation(), entropyproj_limiter=NodewiseScaledExtrapolation())
    res = {}
    for name, lim in limiters.items():
        rep = {}
        for refsem in (True, False):
            kw = gauss if name.startswith("gauss") else {}
            param, ic, bcf = problems.double_mach_reflection(N=3, Kx=480, Ky=120, T=0.2, rhs_limiter=lim,
                                                             reference_semantics=refsem, **kw)
            md, bc, desc, U0 = build_descriptor(param, ic, bcf)
            sec, U, n = _timed_alone(param, md, desc, U0, args.warmup, args.steps, tune=not args.no_autotune)
            rep["reference_semantics" if refsem else "intended"] = {
                "dof_stage_per_s": desc.K * desc.Nq * 3 * n / sec, "ms_per_step": 1e3 * sec / n, "steps": n,
                "min_rho": float(np.reshape(U, (-1, 4))[:, 0].min())}
        res[name] = rep
    print(json.dumps({"metric": METRIC, "unit": UNIT, "workload": "double Mach reflection 480x120, N=3, FP64, per limiter",
                      "data": "synthetic", "report": res}), flush=True)


def run_line_report(args):
    """1D Euler (the Line path, CompressibleEulerIdealGas{Dim1}) on the reference's 1D
    configurations and on a long line: GPU seconds per SSP-RK3 step (CUDA events around the
    host-driven steps, so launch gaps and the per-step dt read-back are included) against
    the FP64 oracle on every host core for the same workload."""
    import torch

    from p2de import problems
    from p2de.types import LobattoCollocation, NoEntropyProjectionLimiter

    torch.cuda.set_device(0)
    lgl = dict(approximation_basis=LobattoCollocation(), entropyproj_limiter=NoEntropyProjectionLimiter())
    cases = {
        "shu-osher K=64 N=3 (examples/1D/shu-osher.jl: Gauss, scaled extrapolation, positivity)":
            (problems.shu_osher, dict(N=3, K=64, T=1.8)),
        "leblanc K=400 N=5 (leblanc-convergence.jl's largest: LGL, positivity)":
            (problems.leblanc, dict(N=5, K=400, **lgl)),
        "shu-osher K=131072 N=3 (a long line)": (problems.shu_osher, dict(N=3, K=131072, T=1.8)),
    }
    res = {}
    for name, (prob, kw) in cases.items():
        if args.line_case and not name.startswith(args.line_case):
            continue
        param, ic, bcf = prob(**kw)[:3]
        md, bc, desc, U0 = build_descriptor(param, ic, bcf)
        steps = min(args.steps, 200)
        sec, U, n = _timed_alone(param, md, desc, U0, args.warmup, steps, tune=False)
        dofs = desc.K * desc.Nq
        cpu = cpu_baseline(desc, U0, dofs, budget_s=4.0)
        res[name] = {"gpu_dof_stage_per_s": dofs * 3 * n / sec, "gpu_ms_per_step": 1e3 * sec / n, "steps": n,
                     "cpu": cpu, "gpu_over_cpu": (dofs * 3 * n / sec) / cpu["value"],
                     "min_rho": float(np.reshape(U, (-1, 3))[:, 0].min())}
    print(json.dumps({"metric": METRIC, "unit": UNIT, "workload": "1D Euler (Line path), FP64",
                      "data": "synthetic", "report": res}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="dmr",
                    choices=["dmr", "kh256", "batch64", "serve", "mixed-report", "limiter-report", "line-report"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "mixed-acc64"])
    ap.add_argument("--line-case", default="", help="line-report: only the cases whose name starts with this")
    ap.add_argument("--basis", default="lobatto", choices=["lobatto", "gauss"],
                    help="gauss: the DMR step with GaussCollocation + NodewiseScaledExtrapolation")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mesh", default="", help="dmr: KXxKY instead of 480x120 (smaller profiler captures)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--serve-rates", default="20,100,500")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serve-time-scale", type=float, default=0.01)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-max-active", type=int, default=64)
    ap.add_argument("--serve-steps-per-tick", type=int, default=4)
    ap.add_argument("--serve-precision", default="mixed-acc64", choices=["fp64", "mixed", "mixed-acc64"])
    ap.add_argument("--mixed-N", default="3,5")
    ap.add_argument("--T", type=float, default=1.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch64":
        return run_batch64(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "mixed-report":
        return run_mixed_report(args)
    if args.workload == "line-report":
        return run_line_report(args)
    if args.workload == "limiter-report":
        return run_limiter_report(args)

    import torch

    from p2de import abi, roofline
    from p2de import solver as S

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    param, ic, bcf, wdesc = workload(args.workload, args.precision, args.basis, args.mesh)
    md, bc, desc, U0 = build_descriptor(param, ic, bcf)
    nodes = desc.K * desc.Nq
    solver = S.Solver(param, md, desc, device=local)
    lib = solver.lib
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    solver._check(lib.p2de_set_stream(solver.handle, ctypes.c_void_p(stream.cuda_stream)))
    solver.set_Uq(U0)
    epb_default = solver.elements_per_block()[0]
    epb = epb_default if args.no_autotune else solver.autotune()[0]

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # ---- warm-up and timed region (CUDA-graph replay, device-resident state)
    t = c_double(0.0)
    n = c_int64()
    solver._check(lib.p2de_ssp33_advance(solver.handle, args.warmup, byref(t), byref(n)))
    l0 = solver.launch_count()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        solver._check(lib.p2de_ssp33_advance(solver.handle, args.steps, byref(t), byref(n)))
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = solver.launch_count() - l0
    steps_done = n.value
    if dist is not None:
        mt = torch.tensor([ms], device="cuda")
        dist.all_reduce(mt, op=dist.ReduceOp.MAX)
        ms = float(mt.item())
    value = world * nodes * 3 * steps_done / (ms * 1e-3)
    clocks = clk.summary()

    # ---- per-kernel timing and the data-dependent work counter (same workload, live)
    cnt = (c_uint64 * 1)()
    solver._check(lib.p2de_read_counters(solver.handle, cnt, 1))
    prof_steps = 5
    kms = (c_double * 3)()
    solver._check(lib.p2de_profile_steps(solver.handle, prof_steps, byref(t), kms))
    solver._check(lib.p2de_read_counters(solver.handle, cnt, 1))
    quad_per_launch = cnt[0] / (3 * prof_steps)
    flops_a = roofline.stage_a_flops(param.N, desc.K, quad_per_launch)
    peak = c_double()
    probe = fma_probe_library()
    rc = probe.p2de_probe_fma_peak(local, 1, byref(peak))
    if rc != 0:
        raise RuntimeError(f"FMA probe failed with status {rc}")
    achieved = flops_a / (kms[0] * 1e-3) / 1e12

    # ---- end-to-end through the public ABI with host buffers
    pinned = torch.empty(nodes * 4, dtype=torch.float64, pin_memory=True)
    host = pinned.numpy()
    solver._check(lib.p2de_get_field(solver.handle, abi.FIELD_UQ, 1, abi.dptr(host)))
    te = c_double(t.value)
    dte = c_double()
    barrier()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.e2e_steps):
        solver._check(lib.p2de_set_Uq(solver.handle, abi.dptr(host)))
        solver._check(lib.p2de_ssp33_step(solver.handle, byref(te), byref(dte)))
        solver._check(lib.p2de_get_field(solver.handle, abi.FIELD_UQ, 1, abi.dptr(host)))
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3)
    if dist is not None:
        mt = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(mt, op=dist.ReduceOp.MAX)
        ms_e2e = float(mt.item())
    e2e_value = world * nodes * 3 * args.e2e_steps / (ms_e2e * 1e-3)
    mins = np.zeros(6)
    solver._check(lib.p2de_stage_minima(solver.handle, abi.dptr(mins)))

    # ---- the same workload under the intended limiter semantics (the 5-tuple bound read
    #      with five names, so the positivity and cell-entropy limiting is active rather than
    #      the first-order scheme the reference's 4-name destructuring gives): same launch
    #      shape, warm-up and step count, CUDA events on the launching stream
    intended = None
    if param.reference_semantics:
        from dataclasses import replace as dc_replace

        p_int = dc_replace(param, reference_semantics=False)
        d_int = S.make_descriptor(p_int, md, bc)
        si = S.Solver(p_int, md, d_int, device=local)
        si._check(lib.p2de_set_stream(si.handle, ctypes.c_void_p(stream.cuda_stream)))
        si.set_Uq(U0)
        si.set_elements_per_block(epb)
        si.set_layout(solver.layout())
        ti, ni = c_double(0.0), c_int64()
        si._check(lib.p2de_ssp33_advance(si.handle, args.warmup, byref(ti), byref(ni)))
        barrier()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record(stream)
        si._check(lib.p2de_ssp33_advance(si.handle, args.steps, byref(ti), byref(ni)))
        e5.record(stream)
        torch.cuda.synchronize()
        ms_int = e4.elapsed_time(e5)
        if dist is not None:
            mt = torch.tensor([ms_int], device="cuda")
            dist.all_reduce(mt, op=dist.ReduceOp.MAX)
            ms_int = float(mt.item())
        mins_i = np.zeros(6)
        si._check(lib.p2de_stage_minima(si.handle, abi.dptr(mins_i)))
        intended = {
            "value": world * nodes * 3 * ni.value / (ms_int * 1e-3),
            "unit": UNIT,
            "ms_per_step": ms_int / max(ni.value, 1),
            "steps": ni.value,
            "limiter": "positivity + cell entropy, bound tuple read with five names (reference_semantics = 0)",
            "min_rho_rhoe_last_step": [float(mins_i[4]), float(mins_i[5])],
        }
        si.close()

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(desc, U0, nodes)
        bytes_ab = roofline.stage_bytes(param.N, desc.K)
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": steps_done,
            "warmup": args.warmup,
            "ms_per_step": ms / steps_done,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else f"f64+f32 ({args.precision})",
            "data": "synthetic",
            "config": {
                "workload": wdesc,
                "elements": desc.K,
                "nodes": nodes,
                "precision": args.precision,
                "parallelism": f"replicas x{world}" if world > 1 else "single solve",
                "l2": "working set per step > L2 (stage data ~%.0f MB per launch)" % (bytes_ab["stage_a"] / 1e6),
                "timing": "CUDA-graph replay of whole steps, CUDA events on the launching stream",
                "elements_per_block": epb,
                "elements_per_block_source": "default" if args.no_autotune else f"autotuned (default {epb_default})",
                "layout": ["flat", "lines per warp"][solver.layout()],
                "threads_per_block_stage_a": solver.threads_per_block(),
            },
            "e2e": {
                "value": e2e_value,
                "unit": UNIT,
                "h2d_bytes_per_step": nodes * 4 * 8,
                "d2h_bytes_per_step": nodes * 4 * 8,
                "steps": args.e2e_steps,
            },
            "gpu_launches": int(launches),
            "clocks": clocks,
            "roofline": {
                "bound": "fp64",
                "kernel": "k_stage_a (low-order RHS, high-order RHS, limiter bounds)",
                "achieved": achieved,
                "peak": peak.value,
                "unit": "TFLOP/s",
                "frac": achieved / peak.value,
                "traffic": KERNEL_A_TRAFFIC_BYTES,
                "fp64_pipe_busy_ncu": KERNEL_A_FP64_PIPE_BUSY,
                "algorithmic_flops_per_launch": flops_a,
                "quad_solves_per_launch": quad_per_launch,
                "ms_per_launch": kms[0],
                "ms_per_launch_stage_b": kms[1],
                "stage_b_hbm_gbs": bytes_ab["stage_b"] / (kms[1] * 1e-3) / 1e9,
                "peak_source": "libp2de_probe.so p2de_probe_fma_peak: FP64 FMA chains on this GPU in this run (MEASURED_PEAKS.json has no FP64 figure)",
            },
            "min_rho_rhoe_last_step": [float(mins[4]), float(mins[5])],
            "intended_semantics": intended,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    solver.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
