#!/usr/bin/env python
"""Benchmark: tricubic 'both'-mode queries/s on a 256^3 dipole vector field.

One step = the whole interpolation job on one batch: construct the
interpolant from the N x 6 field (ingest, per-mode fields) and evaluate
1.01e7 query rows (1e7 uniform in the interpolation volume + 1e5 just
outside it, which must come back NaN), in the precision under test
(default 'mixed': split float32 evaluation with a float64 index step).
The float64 drop-in path is timed beside it.

value: queries/s with the field and queries already resident in HBM.
e2e:   the same job through the public API with host (pinned NumPy) buffers:
       field + queries host->device and comps/norms/grads device->host inside
       the timed region.
Inputs are larger than L2 (field 805 MB, queries 242 MB), so no flush.

Multi-GPU: replicas (every rank builds the full field and evaluates its own
1.01e7 queries; no collective): scaling "weak", value = all ranks' queries /
max-over-ranks time.

--impl reference times the reference's own code (its module byte-compiled
into oracle/_ref by oracle/ref_build.py; the oracle port where that is
absent) on all host cores: worker processes split the 1.01e7-query job by
cell range, each constructing from the whole field, and every step runs one
cold part of the job (its own cells' lazy solves included) on every worker.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tricubic queries/s at 256³ 'both': split-BF16 vs FP64 GPU at ≤1e-6 rel err"
N_IN, N_OUT = 10_000_000, 100_000
GRID = (256, 256, 256)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--strategy", default="auto", choices=["auto", "otf", "table"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="skip the c0/c2/c3/c4 keys of the default line")
    p.add_argument("--grid", type=int, default=GRID[0], help=argparse.SUPPRESS)   # CPU tests of the reference arm
    p.add_argument("--kernel-only", action="store_true", help="time only the query kernel (profiling)")
    p.add_argument("--workload", default=None, choices=["c0", "c2", "c3", "c4", "traj", "csv"],
                   help="measure one of the other seeded configurations and print its own JSON line: "
                        "c0 = 41^3 scalar, 1e5 queries; c2 = 4D 64^3x32 scalar, 1e7 queries; c3 = 512 batched "
                        "scalar fields in one persistent launch / CUDA graph; c4 = differentiable 128^3 "
                        "float32 field, 1e6 queries, forward + backward; traj = 1e6 particles, 100 RK4 steps "
                        "through the 256^3 'both' field; csv = the 256^3 'both' field as a savetxt '%%.18e' "
                        "CSV file (2.6 GB) read as np.genfromtxt(delimiter=',') does")
    p.add_argument("--profile", default=None,
                   choices=["step", "small", "small-table", "small-fp64", "small-coef", "small-4d", "small-batched",
                            "small-adjoint", "small-csv", "small-scalar", "small-traj"],
                   help="run a fixed workload for an ncu capture and exit (no timing, no JSON): "
                        "'step' = two full bench steps; 'small*' = 160^3 dipole field, 2.02e6 queries; "
                        "'small-coef' = 96^3 table solve; 'small-4d' = 40^3x12 scalar, 2e6 queries (on the fly "
                        "and table); 'small-batched' = 64 scalar fields; 'small-adjoint' = 96^3 scalar, 2e6 "
                        "queries forward + backward; 'small-csv' = the 128^3 'both' field file (324 MB) "
                        "parsed twice; 'small-scalar' = 160^3 scalar and 160^3 vector fields, 2e6 queries "
                        "each; 'small-traj' = 2e5 particles x 20 RK4 steps in the 160^3 'both' field")
    return p.parse_args()


EVAL_SMALL_TRAFFIC = 246.96e6  # dram read + write of eval_binc_kernel<4> on the 160^3 case (ncu capture)
# the same capture's shared-memory load wavefronts and warp instructions per query: the kernel's two
# on-chip limits, turned into time bounds for the launch at one wavefront per SM per clock and at one
# warp instruction per scheduler per clock
EVAL_SMALL_WAVEFRONTS_PER_QUERY = 30.584051e6 / 2.02e6
EVAL_SMALL_WARP_INSTR_PER_QUERY = 104.498808e6 / 2.02e6
# dram read + write of eval_tab_coop_kernel<4, mixed> per query: 1.902 GB for 2.02e6 queries on the
# 160^3 table (3.94M cells; ncu capture)
TAB_SMALL_TRAFFIC_PER_QUERY = (1.777388e9 + 0.124713e9) / 2.02e6
# dram read + write of parse_kernel per byte of text: 444.0 MB for the 128^3 field file (324.0 MB; ncu capture)
CSV_PARSE_TRAFFIC_PER_BYTE = (366.16e6 + 77.83e6) / 324.01e6


def on_chip_bounds(kt, nq, clks):
    """Time bounds of the evaluation kernel's on-chip limits for nq queries at
    the median SM clock sampled during the run, from the per-query counts of
    its ncu capture, and the fraction of the measured kernel time kt (s)
    each accounts for."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    hz = 1e6 * (clks.get("sm_mhz") or 2070.0)
    smem = EVAL_SMALL_WAVEFRONTS_PER_QUERY * nq / (sms * hz)
    issue = EVAL_SMALL_WARP_INSTR_PER_QUERY * nq / (sms * 4 * hz)
    return {"shared_memory": {"per_query": EVAL_SMALL_WAVEFRONTS_PER_QUERY, "unit": "wavefronts",
                              "bound_ms": 1000 * smem, "frac": smem / kt},
            "issue": {"per_query": EVAL_SMALL_WARP_INSTR_PER_QUERY, "unit": "warp instructions",
                      "bound_ms": 1000 * issue, "frac": issue / kt},
            "source": "ncu capture of the same kernel on the 160^3 case (bench.py --profile small)"}


def run_profile(args):
    """Fixed workloads for ncu captures (no timing, no JSON)."""
    import torch
    from arbinterp_gb300 import tricubic, synth
    dev = torch.device("cuda")
    if args.profile == "step":
        field, q, lo, hi, h = make_workload(dev)
        for _ in range(2):
            tricubic(field, "quiet", mode="both", precision=args.precision, strategy=args.strategy).Query(q)
    elif args.profile == "small-4d":
        from arbinterp_gb300 import quadcubic
        field = synth.moving_gaussian_field4(n=(40, 40, 40, 12), device=dev)
        for prec in ("mixed", "fp64"):
            for strat in ("otf", "table"):
                o = quadcubic(field, "quiet", precision=prec, strategy=strat)
                q = synth.uniform_queries([float(v) for v in o._lo], [float(v) for v in o._hi], 2_000_000, 0,
                                          [float(v) for v in o._h], seed=3, device=dev)
                o.Query(q)
    elif args.profile == "small-csv":
        from arbinterp_gb300 import fieldfile
        text = synth.field_csv_text((128, 128, 128), 3, seed=5, device=dev)
        for _ in range(2):
            fieldfile.parse_device_text(text, text.numel())
    elif args.profile == "small-batched":
        from arbinterp_gb300.batched import BatchedTricubic
        fields, qs, counts = [], [], []
        for f, nqf, seed in synth.batched_fields(n_fields=64, device=dev):
            o = tricubic(f, "quiet")
            fields.append(f)
            qs.append(synth.uniform_queries([float(v) for v in o._lo], [float(v) for v in o._hi], nqf, 0,
                                            [float(v) for v in o._h], seed=seed % (1 << 30), device=dev))
            counts.append(nqf)
        b = BatchedTricubic(fields, precision="mixed")
        b.tile_rows, b.table_ratio = 1024, None      # fixed plan: no tuning launches in the capture
        b._apply_strategy(counts, None)
        q = torch.cat(qs)
        for _ in range(2):
            b.query(q, counts)
    elif args.profile == "small-adjoint":
        from arbinterp_gb300.autograd import TricubicField
        rows = synth.gaussian_field3(n=(96, 96, 96), seed=7, device=dev)
        for prec in ("mixed", "fp64"):
            fld = TricubicField(rows, precision=prec)
            q = synth.uniform_queries([float(v) for v in fld.interp._lo], [float(v) for v in fld.interp._hi],
                                      2_000_000, 0, [float(v) for v in fld.interp._h], seed=8, device=dev)
            v = fld.initial_values().clone().requires_grad_(True)
            qq = q.clone().requires_grad_(True)
            val, _ = fld(v, qq)
            torch.nan_to_num(val).sum().backward()
    elif args.profile == "small-scalar":
        # one (hi, lo) field and three float32 components: the 3D one-field / vector bin tiles
        for field, kw in ((synth.gaussian_field3(n=(160, 160, 160), h=(0.01, 0.012, 0.008), seed=5, device=dev), {}),
                          (synth.dipole_field3(n=(160, 160, 160), seed=1, device=dev), {"mode": "vector"})):
            o = tricubic(field, "quiet", precision="mixed", strategy="otf", **kw)
            q = synth.uniform_queries([float(v) for v in o._lo], [float(v) for v in o._hi], 2_000_000, 20_000,
                                      [float(v) for v in o._h], seed=3, device=dev)
            for _ in range(2):
                o.Query(q.clone())
    elif args.profile == "small-traj":
        field = synth.dipole_field3(n=(160, 160, 160), seed=1, device=dev)
        o = tricubic(field, "quiet", mode="both", precision="mixed")
        g0 = torch.Generator(device=dev).manual_seed(13)
        lo = torch.tensor([float(v) for v in o._lo], device=dev)
        hi = torch.tensor([float(v) for v in o._hi], device=dev)
        x0 = lo + (hi - lo) * (0.25 + 0.5 * torch.rand((200_000, 3), generator=g0, device=dev, dtype=torch.float64))
        v0 = 1e-3 * torch.randn((200_000, 3), generator=g0, device=dev, dtype=torch.float64)
        for _ in range(2):
            o.trajectories(x0, v0, 0.05, 20, coef=-1e-4)
    elif args.profile == "small-coef":
        # 96^3 'both' field: 804k cells x 4 fields x 64 float32 coefficients = 0.82 GB table
        field = synth.dipole_field3(n=(96, 96, 96), seed=1, device=dev)
        o = tricubic(field, "quiet", mode="both", precision=args.precision, strategy="table")
        for _ in range(2):
            o.allCoeffs()
    else:
        prec = "fp64" if args.profile == "small-fp64" else "mixed"
        strategy = "table" if args.profile == "small-table" else "otf"
        field = synth.dipole_field3(n=(160, 160, 160), seed=1, device=dev)
        o = tricubic(field, "quiet", mode="both", precision=prec, strategy=strategy)
        q = synth.uniform_queries([o.xIntMin, o.yIntMin, o.zIntMin], [o.xIntMax, o.yIntMax, o.zIntMax],
                                  2_000_000, 20_000, [o.hx, o.hy, o.hz], seed=3, device=dev)
        for _ in range(2):
            o.Query(q)
    torch.cuda.synchronize()
    print("profile workload done")


# ---------------------------------------------------------------- other configurations
def _normwise(a, b):
    import torch
    m = torch.isfinite(b).all(1)
    return [float(x) for x in (a[m] - b[m]).abs().amax(0) / b[m].abs().amax(0).clamp_min(1e-300)]


def run_workload(args):
    """One JSON line for one of the other seeded configurations."""
    print(json.dumps(workload_line(args.workload, args.steps, args.warmup)), flush=True)


def _vs_oracle(out, want, inds=None, want_inds=None):
    """Normwise errors of (norms, grads[, comps]) device outputs against the
    oracle's dict, plus bit-exact NaN masks and cell indices."""
    import numpy as np
    res = {}
    for name, got in out.items():
        g = got.cpu().numpy().reshape(len(got), -1)
        w = np.asarray(want[name]).reshape(len(g), -1)
        m = np.isfinite(w).all(1)
        res[name] = [float(x) for x in np.abs(g[m] - w[m]).max(0) / np.maximum(np.abs(w[m]).max(0), 1e-300)]
        res[name + "_nan_mask_equal"] = bool(np.array_equal(np.isnan(g), np.isnan(w)))
    if inds is not None:
        res["indices_bitexact"] = bool(np.array_equal(inds.cpu().numpy(), want_inds))
    return res


def workload_line(name, steps, warmup):
    """Seeded stand-ins for the other configurations.  Mixed precision is
    compared with the float64 GPU path, and both with the CPU oracle on the
    whole query set (c0) or a bounded sample of it (c2: 1e5 rows; c3: 16 of
    the fields; c4: 1e5 rows, forward values and the adjoint)."""
    import numpy as np
    import torch
    from arbinterp_gb300 import tricubic, quadcubic, synth, _lib
    _lib.lib()
    dev = torch.device("cuda")
    gpu_index = torch.cuda.current_device()

    class _A:
        pass
    args = _A()
    args.workload, args.steps, args.warmup = name, steps, warmup
    line = {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
            "scaling": "weak", "vs_baseline": None, "higher_is_better": True, "workload": args.workload}
    if args.workload in ("c0", "c2"):
        if args.workload == "c0":
            field = synth.gaussian_field3(n=(41, 41, 41), h=(0.1, 0.12, 0.08), seed=0, device=dev)
            cls, dim, nin, nout = tricubic, 3, 100_000, 1_000
            desc = "tricubic 41^3 scalar (8 Gaussians), construct + 1.01e5 queries (1e3 outside)"
        else:
            field = synth.moving_gaussian_field4(device=dev)
            cls, dim, nin, nout = quadcubic, 4, 10_000_000, 0
            desc = "quadcubic 64^3 x 32 scalar (6 moving Gaussians), construct + 1e7 queries"
        o64 = cls(field, "quiet")
        lo = [float(v) for v in o64._lo]
        hi = [float(v) for v in o64._hi]
        q = synth.uniform_queries(lo, hi, nin, nout, [float(v) for v in o64._h], seed=5, device=dev)
        nq = q.shape[0]
        res = {}
        for prec in ("fp64", "mixed"):
            for strat in (("otf", "table") if args.workload == "c2" else ("auto",)):
                def step():
                    return cls(field, "quiet", precision=prec, strategy=strat).Query(q)
                with ClockSampler(gpu_index) as clk:
                    dt = cuda_time(step, args.steps, args.warmup)
                out = step()
                res[(prec, strat)] = {"value": nq * args.steps / dt, "unit": "queries/s",
                                      "ms_per_step": 1000 * dt / args.steps, "clocks": clk.summary(),
                                      "_out": out}
        ref = res[("fp64", "otf" if args.workload == "c2" else "auto")]["_out"]
        for k, r in res.items():
            got = r.pop("_out")
            r["max_rel_err_vs_fp64"] = {"norms": _normwise(got[0], ref[0]), "grads": _normwise(got[1], ref[1])}
        head = res[("mixed", "otf" if args.workload == "c2" else "auto")]
        # against the CPU oracle (c0: every query; c2: the first 1e5 rows)
        from oracle.arb_oracle import OracleQuadcubic, OracleTricubic
        ns = nq if args.workload == "c0" else 100_000
        qs_ = q[:ns]
        orc = (OracleTricubic if args.workload == "c0" else OracleQuadcubic)(field.cpu().numpy())
        want = orc.query(qs_.cpu().numpy().copy())
        vs_or = {}
        for (p_, s_) in res:
            ob = cls(field, "quiet", precision=p_, strategy=s_)
            nrm, grd = ob.Query(qs_.clone())
            vs_or[f"{p_}/{s_}"] = _vs_oracle({"norms": nrm, "grads": grd}, want, ob._last_inds, want["inds"])
        line.update({"metric": f"{args.workload}: queries/s, construct + query", "value": head["value"],
                     "unit": "queries/s", "ms_per_step": head["ms_per_step"], "dtype": "f32",
                     "config": {"workload": desc, "precision": "mixed"},
                     "paths": {f"{p}/{s}": v for (p, s), v in res.items()},
                     "vs_oracle": {"rows": ns, **vs_or}})
    elif args.workload == "c3":
        from arbinterp_gb300.batched import BatchedTricubic
        fields, qs, counts = [], [], []
        for f, nqf, seed in synth.batched_fields(device=dev):
            o = tricubic(f, "quiet")
            fields.append(f)
            qs.append(synth.uniform_queries([float(v) for v in o._lo], [float(v) for v in o._hi], nqf, 0,
                                            [float(v) for v in o._h], seed=seed % (1 << 30), device=dev))
            counts.append(nqf)
            del o
        q = torch.cat(qs)
        del qs
        nq = q.shape[0]
        out = {}
        for prec in ("mixed", "fp64"):
            b = BatchedTricubic(fields, precision=prec)
            b.tune(q, counts)
            qbuf = q.clone()
            graph, outs = b.capture(qbuf, counts)
            with ClockSampler(gpu_index) as clk:
                dt = cuda_time(graph.replay, args.steps, args.warmup)
            out[prec] = {"value": nq * args.steps / dt, "ms_per_step": 1000 * dt / args.steps,
                         "tile_rows": b.tile_rows, "table_ratio": b.table_ratio, "clocks": clk.summary(),
                         "_o": [t.clone() for t in outs]}
            del b, graph, outs
        off = np.concatenate([[0], np.cumsum(counts)])
        per_field = []
        for k in range(len(fields)):
            sl = slice(int(off[k]), int(off[k + 1]))
            e = [max(_normwise(a[sl], r[sl])) for a, r in zip(out["mixed"]["_o"], out["fp64"]["_o"])]
            per_field.append(max(e))
        # against the CPU oracle: every 32nd field, at most 2e4 of its rows
        from oracle.arb_oracle import OracleTricubic
        vs_or = {"fields": 0, "rows": 0, "fp64_max": 0.0, "mixed_max": 0.0, "nan_masks_equal": True}
        for k in range(0, len(fields), 32):
            sl = slice(int(off[k]), int(min(off[k + 1], off[k] + 20_000)))
            want = OracleTricubic(fields[k].cpu().numpy()).query(q[sl].cpu().numpy().copy())
            for prec in ("fp64", "mixed"):
                e = _vs_oracle({"norms": out[prec]["_o"][0][sl], "grads": out[prec]["_o"][1][sl]}, want)
                vs_or[prec + "_max"] = max(vs_or[prec + "_max"], max(e["norms"] + e["grads"]))
                vs_or["nan_masks_equal"] &= e["norms_nan_mask_equal"] and e["grads_nan_mask_equal"]
            vs_or["fields"] += 1
            vs_or["rows"] += sl.stop - sl.start
        for v in out.values():
            v.pop("_o")
        line["vs_oracle"] = vs_or
        line.update({"metric": "c3: batched queries/s (one persistent launch, CUDA graph replay)",
                     "value": out["mixed"]["value"], "unit": "queries/s",
                     "ms_per_step": out["mixed"]["ms_per_step"], "dtype": "f32",
                     "config": {"workload": f"{len(fields)} scalar fields, edges 16-128 log-uniform, "
                                            f"{nq} queries in total (1e3-1e6 per field)",
                                "precision": "mixed"},
                     "paths": out,
                     "per_field_max_rel_err_vs_fp64": {"max": max(per_field), "median": float(np.median(per_field))}})
    elif args.workload == "traj":
        field = synth.dipole_field3(n=GRID, seed=1, device=dev)
        g0 = torch.Generator(device=dev).manual_seed(13)
        res = {}
        for prec in ("mixed", "fp64"):
            o = tricubic(field, "quiet", mode="both", precision=prec)
            lo = torch.tensor([float(v) for v in o._lo], device=dev)
            hi = torch.tensor([float(v) for v in o._hi], device=dev)
            x0 = lo + (hi - lo) * (0.25 + 0.5 * torch.rand((1_000_000, 3), generator=g0, device=dev,
                                                          dtype=torch.float64))
            v0 = 1e-3 * torch.randn((1_000_000, 3), generator=g0, device=dev, dtype=torch.float64)
            nsteps, dt = 100, 0.05

            def run():
                return o.trajectories(x0, v0, dt, nsteps, coef=-1e-4)
            with ClockSampler(gpu_index) as clk:
                t = cuda_time(run, max(1, args.steps // 5), 1)
            xs, _ = run()
            res[prec] = {"value": 1_000_000 * nsteps * max(1, args.steps // 5) / t, "unit": "particle-steps/s",
                         "ms_per_step": 1000 * t / max(1, args.steps // 5), "lost": o.lost, "clocks": clk.summary(),
                         "_x": xs}
        m = torch.isfinite(res["fp64"]["_x"]).all(1) & torch.isfinite(res["mixed"]["_x"]).all(1)
        dd = (res["mixed"]["_x"][m] - res["fp64"]["_x"][m]).abs().amax(1)
        # trajectories near the dipoles are chaotic (steep |B|): report quantiles, not just the worst
        dx = {q_: float(torch.quantile(dd.float(), q_)) for q_ in (0.5, 0.9, 0.99)}
        dx["max"] = float(dd.max())
        for v in res.values():
            v.pop("_x")
        line.update({"metric": "traj: RK4 particle-steps/s (4 field evaluations per step)",
                     "value": res["mixed"]["value"], "unit": "particle-steps/s",
                     "ms_per_step": res["mixed"]["ms_per_step"], "dtype": "f32",
                     "config": {"workload": "1e6 particles x 100 RK4 steps in the 256^3 dipole |B| field "
                                            "(x'' = -1e-4 grad|B|)", "precision": "mixed"},
                     "paths": res, "position_diff_mixed_vs_fp64_quantiles": dx})
    elif args.workload == "csv":
        line.update(csv_workload(args, dev, gpu_index))
    else:  # c4
        from arbinterp_gb300.autograd import TricubicField
        # float32 samples; both precisions get the same (float64) geometry
        rows = synth.gaussian_field3(n=(128, 128, 128), h=(0.1, 0.12, 0.08), seed=7, device=dev,
                                     dtype=torch.float32).to(torch.float64)
        f64 = TricubicField(rows, precision="fp64")
        lo = [float(v) for v in f64.interp._lo]
        hi = [float(v) for v in f64.interp._hi]
        q = synth.uniform_queries(lo, hi, 1_000_000, 0, [float(v) for v in f64.interp._h], seed=8, device=dev)
        v64 = f64.initial_values()
        with torch.no_grad():
            truth, _ = f64(v64, q)
        gen = torch.Generator(device=dev).manual_seed(9)
        target = truth + 1e-3 * torch.randn(truth.shape, generator=gen, device=dev, dtype=truth.dtype)
        # rows whose cell index passes the last cell (float32 axes are not exactly evenly spaced, so
        # floor((q - IntMin) / h) can reach the upper face; the reference raises IndexError there)
        # come back NaN and are left out of the loss
        keep = torch.isfinite(truth)
        res = {}
        for prec in ("mixed", "fp64"):
            fld = TricubicField(rows, precision=prec) if prec == "mixed" else f64
            vals = fld.initial_values().to(torch.float32 if prec == "mixed" else torch.float64)

            def fwd_bwd():
                v = vals.clone().requires_grad_(True)
                qq = q.clone().requires_grad_(True)
                val, _ = fld(v, qq)
                diff = torch.where(keep, val - target.to(val.dtype), torch.zeros_like(val))
                loss = (diff * diff).sum()
                loss.backward()
                return v.grad, qq.grad
            with ClockSampler(gpu_index) as clk:
                dt = cuda_time(fwd_bwd, args.steps, args.warmup)
            gv, gq = fwd_bwd()
            res[prec] = {"value": q.shape[0] * args.steps / dt, "ms_per_step": 1000 * dt / args.steps,
                         "clocks": clk.summary(), "_g": (gv.double(), gq.double())}
        # central differences of the (quadratic) loss on 1000 random grid values, float64
        idx = torch.randperm(v64.numel(), generator=torch.Generator().manual_seed(10))[:1000].to(dev)

        def loss64(v):
            with torch.no_grad():
                val, _ = f64(v, q)
                return float(((val - target)[keep] ** 2).sum())
        g64 = res["fp64"]["_g"][0]
        gscale = float(g64[torch.isfinite(g64)].abs().max())
        fd_err, fd_nan = [], 0
        for j in idx.tolist():
            eps = 1e-3
            vp, vm = v64.clone(), v64.clone()
            vp[j] += eps
            vm[j] -= eps
            fd = (loss64(vp) - loss64(vm)) / (2 * eps)
            e = abs(fd - float(g64[j])) / max(1e-300, gscale)
            if e == e:
                fd_err.append(e)
            else:
                fd_nan += 1
        gv_m, gq_m = res["mixed"]["_g"]
        gv_d, gq_d = res["fp64"]["_g"]
        m = torch.isfinite(gq_d).all(1)
        for v in res.values():
            v.pop("_g")
        # against the CPU oracle on the first 1e5 rows: forward values, and the
        # adjoint (value gradient of that subset's loss) against the oracle's
        from oracle.arb_oracle import OracleTricubic
        ns = 100_000
        qs_, ks_ = q[:ns], keep[:ns]
        orc = OracleTricubic(rows.cpu().numpy())
        want = orc.query(qs_.cpu().numpy().copy())
        v = v64.clone().requires_grad_(True)
        val, _ = f64(v, qs_)
        dsub = torch.where(ks_, val - target[:ns], torch.zeros_like(val))
        (dsub * dsub).sum().backward()
        dval = (2 * dsub).detach().cpu().numpy()
        g_or = orc.adjoint(qs_.cpu().numpy(), dval)
        g_gpu = v.grad.detach().cpu().numpy()
        line["vs_oracle"] = {
            "rows": ns,
            "fp64_values": _vs_oracle({"norms": val.detach().view(-1, 1)}, want)["norms"][0],
            "adjoint_fp64_max_rel_err": float(np.abs(g_gpu - g_or).max() / np.abs(g_or).max())}
        line.update({"metric": "c4: forward + backward queries/s (loss = sum of squared residuals)",
                     "value": res["mixed"]["value"], "unit": "queries/s",
                     "ms_per_step": res["mixed"]["ms_per_step"], "dtype": "f32",
                     "config": {"workload": "128^3 float32 scalar field (8 Gaussians), 1e6 queries, targets = "
                                            "float64 interpolant + N(0, 1e-3)", "precision": "mixed",
                                "rows_left_out": int((~keep).sum())},
                     "paths": res,
                     "grad_values_fd_check": {"entries": len(fd_err) + fd_nan, "nan_entries": fd_nan,
                                              "max_rel_err": max(fd_err) if fd_err else None,
                                              "truth_nan": int(torch.isnan(truth).sum()),
                                              "grad_nan": int(torch.isnan(g64).sum())},
                     "mixed_vs_fp64_grad": {
                         "values": float((gv_m - gv_d).abs().max() / gv_d.abs().max()),
                         "queries": float((gq_m[m] - gq_d[m]).abs().max() / gq_d[m].abs().max())}})
    return line


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def csv_workload(args, dev, gpu_index):
    """The 256^3 'both' field (16.8M rows x 6 values) as a savetxt '%.18e'
    CSV file, parsed as np.genfromtxt(path, delimiter=',') does.  value:
    text resident in HBM -> float64 table; e2e: host bytes -> pinned staging
    -> device -> table -> host array; checked bit for bit against
    np.genfromtxt on two 1e5-line samples, which also give the CPU baseline."""
    import io

    import numpy as np
    import torch
    from arbinterp_gb300 import fieldfile, genfromtxt, synth
    t0 = time.perf_counter()
    raw = synth.field_csv_text(GRID, 3, seed=5, device=dev)
    nbytes = raw.numel()
    text = torch.empty(fieldfile._padded(nbytes), dtype=torch.uint8, device=dev)
    text[:nbytes] = raw
    del raw
    host = text[:nbytes].cpu().numpy().tobytes()
    gen_s = time.perf_counter() - t0

    def run():
        return fieldfile.parse_device_text(text, nbytes)
    with ClockSampler(gpu_index) as clk:
        t = cuda_time(run, args.steps, args.warmup)
    stats, phases = {}, []
    for _ in range(3):
        tm = {}
        out = fieldfile.parse_device_text(text, nbytes, stats=stats, timing=tm)
        phases.append(tm)
    ph = {k: float(np.median([p[k] for p in phases])) for k in phases[0]}
    nrows, ncols, nlines = stats["nrows"], stats["ncols"], stats["nlines"]
    # bit-exact check against np.genfromtxt on two samples (first lines, middle of the file)
    S = 100_000
    checks, cpu_s, cpu_bytes = [], 0.0, 0
    buf = np.frombuffer(host, dtype=np.uint8)
    for start in (0, nbytes // 2):
        if start:
            start = host.index(b"\n", start) + 1
        win = buf[start:start + 200 * S]
        nl = np.flatnonzero(win == 10)
        chunk = host[start:start + int(nl[S - 1]) + 1]
        r0 = 0 if start == 0 else int(np.count_nonzero(buf[:start] == 10))
        c0 = time.perf_counter()
        ref = np.genfromtxt(io.BytesIO(chunk), delimiter=",")
        cpu_s += time.perf_counter() - c0
        cpu_bytes += len(chunk)
        got = out[r0:r0 + S].cpu().numpy()
        checks.append(bool(np.array_equal(got.view(np.uint64), ref.view(np.uint64))))
    del buf
    # end to end through the public API: host bytes in, host array out
    ke = max(1, args.steps // 3)

    def e2e():
        return genfromtxt(host).cpu()
    e2e()
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(ke):
        e2e()
    torch.cuda.synchronize()
    te = (time.perf_counter() - e0) / ke
    peak, src = measured_peaks()
    alg = nbytes + nrows * ncols * 8 + nlines * 12
    achieved = alg / (ph["parse_ms"] / 1000.0) / 1e9
    return {
        "metric": "csv: field-file bytes/s parsed, np.genfromtxt(delimiter=',') drop-in (bit-exact)",
        "value": nbytes * args.steps / t / 1e9, "unit": "GB/s", "ms_per_step": 1000 * t / args.steps,
        "dtype": "u8->f64", "gpu_launches": 9 * args.steps,
        "config": {"workload": f"256^3 'both' field file: {nrows} rows x {ncols} values, savetxt '%.18e' "
                               f"({nbytes / 1e9:.2f} GB); text resident in HBM (larger than L2)",
                   "rows_per_s": nrows * args.steps / t, "generate_s": gen_s},
        "phases_ms": ph,
        "exact_pass_tokens": stats["nexact"],
        "bit_exact_vs_np_genfromtxt": {"samples": 2, "lines_per_sample": S, "all_equal": all(checks)},
        "roofline": {"bound": "hbm", "kernel": "arb_csv_parse (parse_kernel + exact pass)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": CSV_PARSE_TRAFFIC_PER_BYTE * nbytes, "algorithmic_bytes": alg, "peak_source": src},
        "cpu_baseline": {"value": cpu_bytes / cpu_s / 1e9, "unit": "GB/s", "cores": 1, "kind": "reference",
                         "sample": f"np.genfromtxt(BytesIO, delimiter=',') on 2 x {S} lines "
                                   f"({cpu_bytes / 1e6:.0f} MB) of the same file, one host core"},
        "e2e": {"value": nbytes / te / 1e9, "unit": "GB/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nrows * ncols * 8, "ms_per_step": 1000 * te},
        "clocks": clk.summary(),
    }


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6789.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- workload
def make_workload(device, rank=0, n=GRID[0]):
    """The 256^3 dipole field and its 1.01e7 queries.  n: the grid edge (other
    values only in the CPU tests of the reference arm, with the query count
    scaled by the cell count, so the queries per cell stay the job's)."""
    import torch
    from arbinterp_gb300 import synth
    field = synth.dipole_field3(n=(n, n, n), seed=1, device=device)
    h = 2.0 / (n - 1)
    ax = -1.0 + h * torch.arange(n, dtype=torch.float64)
    lo = [float(ax[1])] * 3
    hi = [float(ax[n - 2])] * 3
    scale = ((n - 3) / (GRID[0] - 3)) ** 3
    q = synth.uniform_queries(lo, hi, int(N_IN * scale), int(N_OUT * scale), [h] * 3, seed=10 + rank,
                              device=device)
    return field, q, lo, hi, [h] * 3


def copy_peaks(dev, nbytes=1 << 29, reps=3):
    """Pinned host <-> device copy rates on this machine (GB/s): H2D and D2H alone,
    and each direction while both run (two streams), best of `reps`."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    d2 = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    h.fill_(1)
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def timed(fn):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return nbytes / best / 1e9

    def both():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    out = {"h2d_gbs": timed(lambda: d.copy_(h, non_blocking=True)),
           "d2h_gbs": timed(lambda: h2.copy_(d2, non_blocking=True)),
           "bidir_gbs_each": timed(both),
           "how": f"pinned torch copies of {nbytes >> 20} MiB, best of {reps}; bidir: both directions at once"}
    del h, h2, d, d2
    return out


def cuda_time(fn, steps, warmup, barrier=None):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if barrier:
        barrier()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(steps):
        fn()
    e.record()
    torch.cuda.synchronize()
    if barrier:
        barrier()
    return s.elapsed_time(e) / 1000.0


# ---------------------------------------------------------------- CPU baseline
# The reference's own code (oracle/_ref: its module byte-compiled by
# oracle/ref_build.py; the oracle port where that file is absent) runs the
# job on the host cores as N worker processes that split the query set:
# every worker constructs its own
# interpolant from the whole 256^3 field (the reference's getFieldParams,
# unchanged), then evaluates, with `Query`, the queries of its share of the
# cells.  Shares are contiguous ranges of the flat cell index (z-slabs), so a
# worker's lazily solved coefficient columns are its own and its memory stays
# near 1/N of the reference's 33 GB of coefficient arrays.  Each share is cut
# into P parts, again by cell range, so every part is cold (its cells are
# solved by its own queries) and has the query density of the whole job; a
# step runs one part on every worker at once.  Out-of-volume rows are dealt
# out round robin.

def _ref_cells(q, lo, hi, h, npos, nc):
    """Flat cell index of each row as the reference computes it (rQuery3,
    ARBInterp.py:463-485: rows outside [IntMin, IntMax] are NaN, then float64
    (q - IntMin) / h, floor, NaN -> nc)."""
    import numpy as np
    idx = np.zeros(len(q))
    bad = np.zeros(len(q), bool)
    stride = 1.0
    for a in range(3):
        bad |= (q[:, a] < lo[a]) | (q[:, a] > hi[a])
        idx += np.floor((q[:, a] - lo[a]) / h[a]) * stride
        stride *= npos[a]
    idx[bad | np.isnan(idx)] = nc
    return np.minimum(idx, nc).astype(np.int64)


REF_CHUNK = 100_000


def _ref_worker(conn, field_path, parts, kind):
    """One worker of the CPU baseline (spawned; see the block comment)."""
    import contextlib
    import io
    import numpy as np
    field = np.load(field_path, mmap_mode="r")
    t0 = time.perf_counter()
    if kind == "reference":
        from oracle import ref_build
        R = ref_build.load()
        with contextlib.redirect_stdout(io.StringIO()):
            o = R.tricubic(field, "quiet", mode="both")
        run = o.Query
    else:
        from oracle.arb_oracle import OracleTricubic
        o = OracleTricubic(np.asarray(field), mode="both")
        run = o.query
    conn.send(time.perf_counter() - t0)
    while True:
        k = conn.recv()
        if k is None:
            break
        t0 = time.perf_counter()
        qk = parts[k]
        for c0 in range(0, len(qk), REF_CHUNK):     # Query in 1e5-row chunks (result-identical)
            run(qk[c0:c0 + REF_CHUNK].copy())
        conn.send(time.perf_counter() - t0)
    conn.close()


def _mem_available_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 64.0


def reference_cpu(field_np, q_np, nparts, run_parts, warm_parts=0, n=GRID[0], kind=None):
    """Run the CPU baseline: construct on every worker, then `warm_parts`
    untimed and `run_parts` timed steps (one part per worker per step).
    Returns a dict of the measurements.  kind: 'reference' (oracle/_ref) or
    'port' (the oracle); by default the reference where it is built."""
    import multiprocessing as mp
    import tempfile
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import ref_build
    if kind is None:
        kind = "reference" if ref_build.available() else "port"
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    # each worker holds the sorted field copy (805 MB), its share of the
    # coefficient arrays and the evaluation temporaries: about 6 GB at most
    nw = max(1, min(cores, 16, int(_mem_available_gb() // 6)))
    ax = np.array(field_np[:n, 2])            # meshgrid('ij') rows: z fastest; the same axis on x and y
    lo, hi, npos = [ax[1]] * 3, [ax[n - 2]] * 3, [n - 3] * 3
    nc = (n - 3) ** 3
    cell = _ref_cells(q_np, lo, hi, [abs(ax[0] - ax[1])] * 3, npos, nc)
    share = np.minimum(cell * nw // nc, nw - 1)
    part = np.minimum((cell * nw * nparts // nc) % nparts, nparts - 1)
    oob = np.flatnonzero(cell >= nc)
    share[oob] = oob % nw
    part[oob] = (oob // nw) % nparts
    parts = [[q_np[(share == w) & (part == k)] for k in range(nparts)] for w in range(nw)]
    tmp = tempfile.mkdtemp(prefix="arb_ref_")
    fpath = os.path.join(tmp, "field.npy")
    np.save(fpath, field_np)
    env_keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = "1"
    ctx = mp.get_context("spawn")
    conns, procs = [], []
    try:
        for w in range(nw):
            a, b = ctx.Pipe()
            p = ctx.Process(target=_ref_worker, args=(b, fpath, parts[w], kind), daemon=True)
            p.start()
            conns.append(a)
            procs.append(p)
        t0 = time.perf_counter()
        con = [c.recv() for c in conns]
        t_con = time.perf_counter() - t0
        steps = []
        for k in range(warm_parts + run_parts):
            t0 = time.perf_counter()
            for c in conns:
                c.send(k)
            for c in conns:
                c.recv()
            steps.append(time.perf_counter() - t0)
        for c in conns:
            c.send(None)
        for p in procs:
            p.join(60)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        for p in procs:
            if p.is_alive():
                p.kill()
        try:
            os.remove(fpath)
            os.rmdir(tmp)
        except OSError:
            pass
    nq_part = [sum(len(parts[w][k]) for w in range(nw)) for k in range(nparts)]
    timed = range(warm_parts, warm_parts + run_parts)
    return {"kind": kind, "workers": nw, "construct_s": t_con, "construct_worker_s": max(con),
            "step_s": steps, "nq_part": nq_part,
            "timed_queries": sum(nq_part[k] for k in timed), "timed_s": sum(steps[k] for k in timed),
            "nparts": nparts}


def cpu_baseline(field_np, q_np, nparts=25, run_parts=3):
    """cpu_baseline of the default line: the reference on all host cores,
    construct plus `run_parts` of the `nparts` parts of the job (a bounded
    sample with the job's query density; every part cold)."""
    r = reference_cpu(field_np, q_np, nparts, run_parts)
    v = r["timed_queries"] / r["timed_s"]
    who = ("the reference's own module (oracle/_ref, byte-compiled, unmodified)" if r["kind"] == "reference"
           else "the oracle port (oracle/_ref absent)")
    return {
        "value": v, "unit": "queries/s", "cores": r["workers"], "kind": r["kind"],
        "sample": (f"{who} in {r['workers']} processes splitting the 1.01e7-query job by cell range; each "
                   f"constructs from the whole 256^3 field ({r['construct_worker_s']:.1f} s, not in the value), then "
                   f"{run_parts} of the job's {nparts} parts ({r['timed_queries']} queries, cold: lazy "
                   f"coefficient solves of their own cells) are timed"),
        "construct_s": r["construct_worker_s"], "step_s": r["step_s"],
    }


def run_reference(args):
    """Reference arm: the reference's own code on all host cores (see the
    CPU-baseline block comment).  The job's queries are cut into warmup +
    steps parts per worker; step k evaluates part k on every worker (cold),
    the last `steps` are timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    field, q, lo, hi, h = make_workload("cpu", n=args.grid)
    field_np, q_np = field.numpy(), q.numpy()
    nparts = args.warmup + args.steps
    r = reference_cpu(field_np, q_np, nparts, args.steps, warm_parts=args.warmup, n=args.grid)
    val = r["timed_queries"] / r["timed_s"]
    whole = r["construct_worker_s"] + sum(r["step_s"])
    who = ("the reference's own module (oracle/_ref, byte-compiled, unmodified)" if r["kind"] == "reference"
           else "the oracle port (oracle/_ref absent)")
    line = {
        "metric": METRIC, "value": val, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * r["timed_s"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": f"tricubic {args.grid}^3 dipole vector field, mode both, {len(q_np)} queries "
                               f"(1% outside the volume), cut into {nparts} parts of equal query density; one part "
                               "per step",
                   "construct_s": r["construct_worker_s"],
                   "whole_job_s": whole, "whole_job_queries_per_s": len(q_np) / whole},
        "cpu_baseline": {"value": val, "unit": "queries/s", "cores": r["workers"], "kind": r["kind"],
                         "sample": f"{who} in {r['workers']} processes splitting the query set by cell range; "
                                   f"each step = one cold part per process; construction "
                                   f"({r['construct_worker_s']:.1f} s) before the steps"},
        "e2e": {"value": val, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm
def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)
    if args.workload:
        return run_workload(args)
    import numpy as np
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    barrier = (lambda: dist.barrier()) if world > 1 else None

    from arbinterp_gb300 import tricubic, _lib
    _lib.lib()
    dev = torch.device("cuda", local)
    field, q, lo, hi, h = make_workload(dev, rank)
    nq = q.shape[0]
    prec, strat = args.precision, args.strategy

    def step_dev():
        o = tricubic(field, "quiet", mode="both", precision=prec, strategy=strat)
        return o.Query(q)

    from arbinterp_gb300.replicas import max_over_ranks as tmax   # replicas: whole-job time = max over ranks

    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0]) if \
        os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else local

    if args.kernel_only:
        o = tricubic(field, "quiet", mode="both", precision=prec, strategy=strat)
        t = cuda_time(lambda: o._run(q, nq, 3, False, False), args.steps, args.warmup)
        print(json.dumps({"kernel_ms": 1000 * t / args.steps}))
        return

    with ClockSampler(gpu_index) as clk:
        dt = cuda_time(step_dev, args.steps, args.warmup, barrier)
    dt = tmax(dt)
    value = world * nq * args.steps / dt

    # The dominant kernel is the evaluation pass over the bin-ordered records
    # (56% of the step in the ncu launch list).  Bin the queries once, then
    # time the evaluation launch alone on the launching stream, with the
    # interleaved output rows the public API uses.
    from arbinterp_gb300 import _lib as LB
    L = LB.lib()
    o = tricubic(field, "quiet", mode="both", precision=prec, strategy=strat)
    o.Query(q.clone())                                   # the plan the timed steps use
    use_tab = bool(o.last_plan["table"])
    o._g.bin_shift = int(o.last_plan.get("bin_shift", 0))
    pc = LB.PREC_MIXED if prec == "mixed" else LB.PREC_FP64
    need = int(L.arb_query_sorted_work_bytes(o._g, pc, nq))
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    f64 = dict(dtype=torch.float64, device=dev)
    rows = torch.empty((nq, 8), **f64)                       # cx cy cz |B| gx gy gz -
    oi = torch.empty(nq, dtype=torch.int64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    rp = rows.data_ptr()
    qo = LB.ArbQueryOut(rp, rp + 24, rp + 32, oi.data_ptr(), None, None, 8, 8, 8)
    sp = torch.cuda.current_stream().cuda_stream
    LB.check(L.arb_query_bin(o._g, pc, q.clone().data_ptr(), nq, 3, 0, qo, ws.data_ptr(), need,
                             st.data_ptr(), sp), "arb_query_bin")
    kt = cuda_time(lambda: L.arb_query_eval_binned(o._g, pc, int(use_tab), nq, qo, ws.data_ptr(), need, sp),
                   5, 2) / 5
    rec = 32 if prec == "mixed" else 48                       # bin-ordered query record
    grid_bytes = o._npts * (20 if prec == "mixed" else 32)    # grid read once (compulsory)
    algo = nq * (rec + 7 * 8) + (nq * 4 * 64 * (4 if prec == "mixed" else 8) if use_tab else grid_bytes)
    kname = ("eval_sorted_kernel<3,4,table>" if use_tab else
             ("eval_binc_kernel<4>" if prec == "mixed" else "eval_sorted_kernel<3,4,fp64>"))
    # DRAM traffic per launch, scaled from the small-case ncu capture of the
    # same kernel (`bench.py --profile small`: EVAL_SMALL_TRAFFIC bytes for
    # 2.02e6 queries on a 160^3 grid whose mixed grid is 81.92 MB), per query
    # plus one read of the grid
    traffic = ((nq * (EVAL_SMALL_TRAFFIC - 81.92e6) / 2.02e6 + grid_bytes)
               if (prec == "mixed" and not use_tab) else None)
    peak, peak_src = measured_peaks()
    achieved = algo / kt / 1e9

    # precision of the mixed path against the float64 GPU path (pinned to the oracle)
    extra = {}
    if not args.no_fp64:
        o64 = tricubic(field, "quiet", mode="both", precision="fp64", strategy="otf")
        t64 = cuda_time(lambda: tricubic(field, "quiet", mode="both", precision="fp64").Query(q),
                        max(2, args.steps // 3), 1)
        t64 = tmax(t64)
        v64 = world * nq * max(2, args.steps // 3) / t64
        ref = o64.Query(q.clone())
        got = o.Query(q.clone())
        errs = {}
        for name, a, b in zip(("comps", "norms", "grads"), got, ref):
            m = torch.isfinite(b).all(1)
            assert torch.equal(torch.isnan(a), torch.isnan(b)), name
            d = (a[m] - b[m]).abs().amax(0) / b[m].abs().amax(0)
            errs[name] = [float(x) for x in d]
        same_inds = bool(torch.equal(o._last_inds, o64._last_inds))
        extra = {"fp64_path": {"value": v64, "unit": "queries/s", "ms_per_step": 1000 * t64 / max(2, args.steps // 3)},
                 "speedup_vs_fp64": value / v64,
                 "max_rel_err_vs_fp64": errs, "indices_bitexact": same_inds}
        # both paths against the CPU oracle on the first 1e5 rows of the 256^3 job
        # (bin-grouped: above the sort threshold)
        if rank == 0:
            from oracle.arb_oracle import OracleTricubic
            ns = 100_000
            want = OracleTricubic(field.cpu().numpy(), mode="both").query(q[:ns].cpu().numpy().copy())
            for pname in ("fp64", "mixed"):
                ob = tricubic(field, "quiet", mode="both", precision=pname, strategy="otf")
                c_, n_, g_ = ob.Query(q[:ns].clone())
                extra[pname + "_vs_oracle"] = _vs_oracle({"comps": c_, "norms": n_, "grads": g_}, want,
                                                         ob._last_inds, want["inds"])
                extra[pname + "_vs_oracle"]["rows"] = ns
                del ob

    # warm query-only throughput (interpolant already constructed)
    tq = cuda_time(lambda: o.Query(q), 5, 2) / 5
    extra["warm_query_only"] = {"value": world * nq / tq, "unit": "queries/s"}

    # the coefficient-table strategy: tensor-core table solve + table evaluation
    if prec == "mixed" and not args.no_fp64:
        ot = tricubic(field, "quiet", mode="both", precision=prec, strategy="table")
        tg = cuda_time(lambda: ot.allCoeffs(), 3, 1) / 3
        tt = cuda_time(lambda: ot.Query(q), 3, 1) / 3
        terrs = {}
        for name, a, b in zip(("comps", "norms", "grads"), ot.Query(q.clone()), ref):
            m = torch.isfinite(b).all(1)
            terrs[name] = [float(x) for x in (a[m] - b[m]).abs().amax(0) / b[m].abs().amax(0)]
        cells = ot.nc
        gemm_bytes = ot._npts * 4 * 8 + cells * 4 * 64 * 4
        gemm_flops = 2.0 * 64 * 64 * 4 * cells
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if \
            os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
        # the table evaluation kernel alone (queries binned once), against the
        # compulsory bytes: each distinct cell's 1 KB block once, the record
        # and the output row of every query
        ws_t = torch.empty(int(L.arb_query_sorted_work_bytes(ot._g, pc, nq)), dtype=torch.uint8, device=dev)
        ot._g.bin_shift = 0
        LB.check(L.arb_query_bin(ot._g, pc, q.clone().data_ptr(), nq, 3, 0, qo, ws_t.data_ptr(), ws_t.numel(),
                                 st.data_ptr(), sp), "arb_query_bin")
        kt_tab = cuda_time(lambda: L.arb_query_eval_binned(ot._g, pc, 1, nq, qo, ws_t.data_ptr(), ws_t.numel(),
                                                           sp), 5, 2) / 5
        cells_hit = int(torch.unique(oi[oi < ot.nc]).numel())
        tab_alg = cells_hit * 4 * 64 * 4 + nq * (32 + 7 * 8)
        tab_ach = tab_alg / kt_tab / 1e9
        del ws_t
        extra["roofline_table_eval"] = {
            "bound": "hbm", "kernel": "eval_tab_coop_kernel<4, mixed>", "kernel_ms": 1000 * kt_tab,
            "achieved": tab_ach, "peak": peak, "unit": "GB/s", "frac": tab_ach / peak,
            "traffic": nq * TAB_SMALL_TRAFFIC_PER_QUERY, "algorithmic_bytes": tab_alg, "peak_source": peak_src,
            "distinct_cells": cells_hit,
            "no_dedup_frac": nq * (4 * 64 * 4 + 32 + 7 * 8) / kt_tab / 1e9 / peak}
        extra["table_path"] = {
            "value": world * nq / (tg + tt), "unit": "queries/s",
            "coef_gemm_ms": 1000 * tg, "table_eval_ms": 1000 * tt,
            "coef_gemm_gbs": gemm_bytes / tg / 1e9,
            "coef_gemm_tflops_algorithmic": gemm_flops / tg / 1e12,
            "coef_gemm_hbm_frac": gemm_bytes / tg / 1e9 / peak,
            "coef_gemm_f16_frac": gemm_flops / tg / 1e12 / peaks.get("bf16_tflops", 1900.0),
            "max_rel_err_vs_fp64": terrs,
            "note": (f"table: {cells} cells x 4 fields x 64 float32 coefficients "
                     f"({cells * 4 * 64 * 4 / 1e9:.1f} GB) per solve; FP16 fixed-point parts, exact accumulation")}
        del ot

    e2e = None
    if not args.no_e2e:
        field_h = torch.empty(field.shape, dtype=field.dtype, pin_memory=True)
        field_h.copy_(field)
        q_h = torch.empty(q.shape, dtype=q.dtype, pin_memory=True)
        q_h.copy_(q)
        fnp, qnp = field_h.numpy(), q_h.numpy()
        last = {}

        def step_host():
            ob = tricubic(fnp, "quiet", mode="both", precision=prec, strategy=strat)
            last["out"] = ob.Query(qnp)
            from arbinterp_gb300 import interp as _ip
            lay = ob._packed_layout() if qnp.shape[0] >= _ip.PIPELINE_MIN_ROWS else ob._row_layout()
            last["rows_bytes"] = lay[0] * 8 * qnp.shape[0]

        te = cuda_time(step_host, max(3, args.steps // 2), 2, barrier)
        te = tmax(te)
        ksteps = max(3, args.steps // 2)
        # the outputs are column views of one row buffer (packed: only the returned columns), copied whole
        d2h = last["rows_bytes"]
        h2d = int(fnp.nbytes + qnp.nbytes)
        cp = copy_peaks(dev)
        # copy roofline: the link moves H2D and D2H bytes at the measured
        # pinned rates; "link" ignores what depends on what, "staged" keeps the
        # job's order (the whole field before any result, then the queries in
        # and the results out at the concurrent per-direction rate)
        link_floor = max(h2d / cp["h2d_gbs"], d2h / cp["d2h_gbs"],
                         (h2d + d2h) / (2 * cp["bidir_gbs_each"])) / 1e6
        staged_floor = (fnp.nbytes / cp["h2d_gbs"] + max(qnp.nbytes, d2h) / cp["bidir_gbs_each"]) / 1e6
        ms_e2e = 1000 * te / ksteps
        e2e = {"value": world * nq * ksteps / te, "unit": "queries/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e,
               "copy_peak": cp, "copy_floor_ms": {"link": link_floor, "staged": staged_floor},
               "copy_frac": {"link": link_floor / ms_e2e, "staged": staged_floor / ms_e2e}}

    # the other seeded configurations, measured in the same run (one GPU)
    if rank == 0 and world == 1 and not args.no_configs:
        skip = ("n_gpus", "steps", "warmup", "data", "scaling", "vs_baseline", "higher_is_better", "workload")
        extra["configs"] = {}
        for wname in ("c0", "c2", "c3", "c4"):
            ln = workload_line(wname, args.steps, args.warmup)
            extra["configs"][wname] = {k: v for k, v in ln.items() if k not in skip}
            torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(field.cpu().numpy(), q.cpu().numpy())

    if rank == 0:
        # this library's kernels per step: ingest (meshgrid-order rows: probe, summary, gather,
        # tile; otherwise those four plus axes init/collect/sort, index, gather, summary) and
        # the query (binned: count, two scan passes, place, evaluate; plain: one)
        clks = clk.summary()
        launches_per_step = ((4 if o.ingest_path == "ordered" else 10) +
                             (5 if o.last_plan.get("binned") else 1))
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": "tricubic 256^3 dipole vector field (16 dipoles outside the box), mode both, "
                                   "construct + 1.01e7 queries (1% outside the volume)",
                       "precision": prec, "strategy": "table" if use_tab else "otf",
                       "plan": o.last_plan,
                       "l2": "inputs larger than L2 (field 805 MB, queries 242 MB); no flush"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                         "kernel_ms": 1000 * kt, "algorithmic_bytes": algo, "peak_source": peak_src,
                         "on_chip": on_chip_bounds(kt, nq, clks) if (prec == "mixed" and not use_tab) else None},
            "clocks": clks,
            "gpu_launches": launches_per_step * args.steps,
            "e2e": e2e, "cpu_baseline": cpu,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
