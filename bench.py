"""Benchmark: MPFA-O Richards fused residual + Jacobian (F+J) on GB300.

One step = one TDyMPFAOSNESFunction + TDyMPFAOSNESJacobian evaluation (the
per-Newton-iteration work of the reference's SNES callbacks) over the
60x220x85 jittered-hex workload (SPE10 model-2 grid, seeded synthetic fields;
see tdycore_gb300/workloads.py).  Inputs (~1.9 GB of setup arrays, the
1.12 M-cell state) are larger than the 129 MB L2, so no flush is needed
between iterations.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line on rank 0.  --impl reference times the CPU restatement
of the reference's F+J (the reference itself needs PETSc/MPI and cannot be
built here) on the host cores with all available threads.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MPFA-O F+J cells/s (% HBM peak); batched solves/s, p99 latency @1e-8 resid"
UNIT = "cells/s"
FALLBACK_HBM_GBS = 6800.0
DT = 1800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            for k in ("hbm_gbs", "hbm_GBs", "hbm"):
                if k in d:
                    return float(d[k]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_workload(host_only=False, grid=None, jacobian_arithmetic="DOUBLE_FLOAT", extra_options=""):
    import tdycore_gb300 as T
    from tdycore_gb300.workloads import spe10_like

    T.options_clear()
    T.options_insert(f"-tdy_jacobian_arithmetic {jacobian_arithmetic} {extra_options}")
    t0 = time.perf_counter()
    if grid:
        nx, ny, nz = grid
        t, U, info = spe10_like(nx, ny, nz, lx=365.76 * nx / 60, ly=670.56 * ny / 220, lz=51.816 * nz / 85)
    else:
        t, U, info = spe10_like()
    t1 = time.perf_counter()
    t.setup(host_only=host_only)
    info["setup_s"] = time.perf_counter() - t1
    log(f"setup: {info['workload']} {t.ncells} cells, nnz {t.nnz}, {time.perf_counter() - t0:.1f} s")
    rng = np.random.default_rng(20261203)
    Uprev = U + rng.normal(0.0, 200.0, U.size)
    return t, U, Uprev, info


def algorithmic_bytes(view):
    """Per-evaluation FP64 payload (index arrays excluded):
    8 * (sum_v R_v C_v  [Trans]  +  sum_v R_v  [gravity term per row]
         + 7 Nc  [P, accum_prev, porosity, Sr, alpha, m, volume]
         + N_bD  [Dirichlet boundary pressures]  + Nc  [R out]  + nnz  [J out])."""
    nbd = int(np.sum(view["bnd_has_value"] * (view["bnd_type"] != 1)))
    return 8 * (int(view["ntrans_total"]) + int(view["nrows_total"]) + 7 * view["ncells"] + nbd + view["ncells"]
                + int(view["nnz"]))


def vertex_kernel_bytes(view):
    """The vertex stage's share of the algorithmic bytes (the formula of
    algorithmic_bytes): its Trans blocks, one gravity coefficient per row and
    the cell pressures, 8 * (sum_v R_v C_v + sum_v R_v + Nc).  The state it
    gathers beyond P and the per-vertex partial sums it hands to the cell
    stage are intermediate data of this implementation, not algorithmic
    bytes."""
    return 8 * (int(view["ntrans_total"]) + int(view["nrows_total"]) + int(view["ncells"]))


def workload_config(info, nc, nnz, world):
    """The workload description, identical in both arms of the bench."""
    return {"workload": info["workload"], "ncells": nc, "nnz_jacobian": nnz, "form": "SNES F+J",
            "seed": info["seed"], "l2": "inputs larger than L2 (no flush)",
            "parallelism": f"replicas x{world}" if world > 1 else "one device"}


def fp64_pipe_from_profile(kernel_ms):
    """FP64 pipe utilisation per kernel from the committed ncu summary
    (sm__pipe_fp64_cycles_active), and its average over one evaluation
    weighted by the live per-kernel durations."""
    f = ROOT / "profiles" / "fp64_pipe.json"
    if not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
    except Exception:
        return None
    per = d.get("pipe_fp64_active_frac", {})
    tot = sum(kernel_ms.get(k, 0.0) for k in per)
    avg = sum(per[k] * kernel_ms.get(k, 0.0) for k in per) / tot if tot > 0 else None
    return {"per_kernel": per, "evaluation_time_weighted": avg, "source": "profiles/fp64_pipe.json",
            "captured_workload": d.get("captured_workload")}


def fp64_flops_per_eval(view):
    """FP64 operations of one evaluation by the vertex/cell decomposition:
    2 per Trans entry (T.P), 2 per (row, internal column, adjacent cell) for J,
    ~24 per row for upwinding and the flux/derivative scalars, and one add per
    gathered partial."""
    v_rows = np.diff(view["v_row_off"]).astype(np.int64)
    nint = view["v_nint"].astype(np.int64)
    tp = 2 * int(view["ntrans_total"])
    jac = int(np.sum(v_rows * nint)) * 4
    rows = 24 * int(view["nrows_total"])
    gather = int(np.sum(nint * nint + nint))
    return tp + jac + rows + gather


def make_oracle(view, Uprev):
    from oracle import Oracle

    t0 = time.perf_counter()
    o = Oracle(view)
    o.snes_presolve(Uprev, DT)
    log(f"oracle ready in {time.perf_counter() - t0:.1f} s")
    return o


def parity_full_size(o, U, R, J):
    """Largest error of the GPU R and J against the oracle at the bench
    workload, in units of the oracle's per-entry error scale (the parity tests
    require <= 1e-12 for R and <= 1e-10 for J), and the norm-wise residual
    error ||R - R_ref||_2 / ||R_ref||_2 (the state is perturbed, far from
    equilibrium)."""
    Rr, Rm = o.snes_function(U, with_mag=True)
    Jr, Jm = o.snes_jacobian(U, with_mag=True)
    tiny = np.finfo(float).tiny
    return (float(np.max(np.abs(R - Rr) / np.maximum(Rm, tiny))),
            float(np.max(np.abs(J - Jr) / np.maximum(Jm, tiny))),
            float(np.linalg.norm(R - Rr) / np.linalg.norm(Rr)))


def newton_config1(start="hydrostatic"):
    """The reference's CPU-runnable case (10x10x10 box over the unit cube,
    top Dirichlet at 101325 Pa, 10 backward-Euler steps of 1800 s): the full
    Newton solve with the GPU residual/Jacobian and with the oracle's, the same
    Newton (PETSc SNESNEWTONLS defaults, direct solve) around both.

    start="hydrostatic" is the case as specified: every cell saturated and in
    equilibrium, so each step needs 0-1 Newton iterations and whether one is
    taken depends on FP64 rounding noise (the per-step initial residual norms
    are reported beside the counts).  start="dry" lowers the initial pressure
    by 60 kPa (unsaturated, van Genuchten S_e ~ 0.45): water infiltrates from
    the top face and the first step takes about 8 Newton iterations before the
    box is back at equilibrium."""
    import tdycore_gb300 as T
    from tdycore_gb300 import driver as D
    from tdycore_gb300.workloads import hydrostatic_box
    from oracle import Oracle

    def run(F, J, presolve, U, rp, ci):
        snes = D.SNESNewtonLS()
        its, f0s, t0 = [], [], time.perf_counter()
        for _ in range(10):
            presolve(U)
            f0s.append(float(np.linalg.norm(F(U))))
            res = snes.solve(F, J, U.copy(), rp, ci)
            if res.reason <= 0:
                raise RuntimeError(f"config-1 Newton failed: reason {res.reason}")
            its.append(res.iterations)
            U = res.x
        return U, its, f0s, time.perf_counter() - t0

    T.options_clear()
    t, U0, info = hydrostatic_box()
    if start == "dry":
        U0 = U0 - 60000.0
    t.setup()
    t.set_dtime(1800.0)
    Ug, its_g, f0_g, tg = run(t.snes_function, t.snes_jacobian, t.presolve, U0, t.rowptr, t.colidx)
    o = Oracle(t.setup_view())
    Uc, its_c, f0_c, tc = run(o.snes_function, o.snes_jacobian, lambda U: o.snes_presolve(U, 1800.0), U0,
                              t.rowptr, t.colidx)
    t.destroy()
    return {"workload": info["workload"] + ("" if start == "hydrostatic" else "_dry_start"), "start": start,
            "steps": 10, "dt_s": 1800.0,
            "gpu_wall_s_per_step": tg / 10, "cpu_oracle_wall_s_per_step": tc / 10,
            "newton_iterations_gpu": its_g, "newton_iterations_oracle": its_c,
            "initial_residual_norm_gpu": f0_g, "initial_residual_norm_oracle": f0_c,
            "final_pressure_max_rel_diff_vs_oracle": float(np.max(np.abs(Ug - Uc) / np.abs(Uc))),
            "note": "GPU F+J through the host C-ABI and the CPU oracle's F+J (1 thread), both inside the same "
                    "host Newton with a sparse direct solve; initial_residual_norm = ||F|| at each step's start"}


def batched_config4(ninst=4096, sample=64, dt=3600.0):
    """Config 4: independent hexahedral subdomains (nx, ny ~ U{1..8}, nz ~
    U{10..100}) in one handle, each advanced one backward-Euler step of
    3600 s to a relative FP64 residual of 1e-8 by the device Newton, batched
    with the FP32 Jacobian and inner solve and batched in plain FP64 (which
    separates the gain of precision from the gain of batching), against the
    same instances solved one by one on the plain FP64 path, timed on a
    sample of them.  Every batched instance is checked against the FP64
    oracle."""
    import torch

    import tdycore_gb300 as T
    from tdycore_gb300.workloads import batched_columns
    from oracle import Oracle

    T.options_clear()
    T.options_insert("-tdy_mpfao_setup_on_device")
    t0 = time.perf_counter()
    tb, U0, info = batched_columns(ninst)
    tb.setup()
    setup_s = time.perf_counter() - t0
    log(f"config 4: {ninst} instances, {tb.ncells} cells, setup {setup_s:.1f} s")
    dev = torch.device("cuda")
    off = np.concatenate([[0], np.cumsum(info["instance_cells"])])
    seg = np.repeat(np.arange(ninst), info["instance_cells"])
    o = Oracle(tb.setup_view())
    o.snes_presolve(U0, dt)
    n0 = np.sqrt(np.bincount(seg, weights=o.snes_function(U0) ** 2, minlength=ninst))

    def batched(fp32):
        # warm-up (inner-solve graph, spmv autotune), then the timed batched solve
        d = torch.tensor(U0, dtype=torch.float64, device=dev)
        tb.backward_euler_step_device(d, dt, fp32=fp32)
        d.copy_(torch.tensor(U0, dtype=torch.float64, device=dev))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        stats, its, rel = tb.backward_euler_step_device(d, dt, fp32=fp32)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t1
        Ub = d.cpu().numpy()
        # FP64 oracle residual of every instance
        F1, M1 = o.snes_function(Ub, with_mag=True)
        n1 = np.sqrt(np.bincount(seg, weights=F1 * F1, minlength=ninst))
        m1 = np.sqrt(np.bincount(seg, weights=M1 * M1, minlength=ninst))
        rel_o = n1 / np.maximum(n0, 1e-300)
        at_floor = n1 <= 1e-11 * m1
        meets = (rel_o <= 1.01e-8) | at_floor
        res = {"solves_per_s": ninst / wall, "batch_wall_s": wall,
               "newton_iterations_max": stats["newton_iterations"],
               "newton_iterations_mean": float(np.mean(its)), "linear_iterations_total": stats["linear_iterations"],
               "converged": stats["converged"], "ended_by_step_test_above_rtol": stats["step_converged"],
               "max_rel_residual_device": stats["max_rel_residual"],
               "phases_s": {"eval_s": stats["eval_s"], "precond_s": stats["precond_s"],
                            "krylov_s": stats["krylov_s"]},
               "fp32_inner_solves_redone_in_fp64": stats["fp64_inner_redo"],
               "oracle_fp64": {"max_rel_residual": float(rel_o.max()),
                               "instances_meeting_1e-8": int(np.sum(meets)),
                               "instances_not_meeting": [int(g) for g in np.nonzero(~meets)[0][:8]],
                               "instances_at_fp64_noise_floor": int(np.sum(at_floor & (rel_o > 1.01e-8)))}}
        return res, Ub

    fp32_res, Ub = batched(True)
    fp64_res, Ub64 = batched(False)
    fp64_res["max_rel_diff_vs_fp32_batch"] = float(np.max(np.abs(Ub64 - Ub) / np.abs(Ub64)))
    del o
    blocks, props = tb._blocks, tb._props
    tb.destroy()
    # one by one, plain FP64, on a sample
    rng = np.random.default_rng(7)
    pick = np.sort(rng.choice(ninst, size=min(sample, ninst), replace=False))
    solve_s, max_diff = 0.0, 0.0
    from tdycore_gb300 import workloads as W

    for b in pick:
        c0, c1 = off[b], off[b + 1]
        T.options_clear()
        t = T.create_richards_mpfao()
        t.set_extruded_meshes([blocks[b]])
        t.set_from_options()
        t.set_permeability_values(props["K"][c0:c1])
        t.set_porosity_values(props["poro"][c0:c1])
        t.set_vangenuchten_values(props["m"][c0:c1], props["alpha"][c0:c1])
        t.set_mualem_values(props["m"][c0:c1])
        t.set_constant_residual_saturation(0.15)
        t.set_water_density_type(T.WATER_DENSITY_CONSTANT)
        ztop = blocks[b][2].max()
        ptop = W.PREF + 998.0 * W.GRAVITY * (0.6 * ztop - ztop) + 2000.0
        t.set_boundary_pressure_type_function(
            lambda x, y, z, zt=ztop: np.where(np.asarray(z) > zt - 1e-9, T.DIRICHLET_BC, T.NEUMANN_BC))
        t.set_boundary_pressure_function(lambda x, y, z, p=ptop: np.full(np.shape(x), p))
        t.setup()
        d1 = torch.tensor(U0[c0:c1], dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        ts = time.perf_counter()
        t.backward_euler_step_device(d1, dt, fp32=False)
        torch.cuda.synchronize()
        solve_s += time.perf_counter() - ts
        max_diff = max(max_diff, float(np.max(np.abs(d1.cpu().numpy() - Ub[c0:c1]) / np.abs(Ub[c0:c1]))))
        t.destroy()
    T.options_clear()
    one_by_one = len(pick) / solve_s
    return {
        "workload": info["workload"], "ninstances": ninst, "ncells": int(off[-1]), "dt_s": dt, "setup_s": setup_s,
        "batched_fp32": fp32_res,
        "batched_fp64": fp64_res,
        "one_by_one_fp64": {"solves_per_s": one_by_one, "sample": int(len(pick)),
                            "max_rel_diff_vs_batched_fp32": max_diff,
                            "note": "the same instances, one handle each, FP64 Jacobian and inner solve; "
                                    "solve calls timed, setup excluded"},
        "speedup_batched_fp32_vs_one_by_one": fp32_res["solves_per_s"] / one_by_one,
        "speedup_batched_fp64_vs_one_by_one": fp64_res["solves_per_s"] / one_by_one,
        "speedup_fp32_vs_fp64_batched": fp32_res["solves_per_s"] / fp64_res["solves_per_s"],
        "note": "batched_* = all instances in one handle, one device Newton solve; oracle_fp64 = ||F(U_new)|| / "
                "||F(U_n)|| per instance from the FP64 oracle (an instance that starts within FP64 resolution of "
                "equilibrium counts when ||F|| is within 1e-11 of its error scale); converged = device residual "
                "met 1e-8, ended_by_step_test_above_rtol = stopped by the step test above it",
    }


def prisms_config3(ntri=200_000, nlayers=40, steps=20, dt=1.0, rotation="vertical", precond="clusters",
                   max_cuts=4, attempt_max_it=20, oracle_threads=0):
    """Config 3: infiltration (1e-7 m/s through the top) into a dry soil on
    Delaunay triangular prisms with per-cell full-tensor K, ``steps``
    intervals of ``dt`` advanced by the device Newton in the mixed form (FP64
    residual, FP32 Jacobian and inner solve), and again, from the same start,
    in plain FP64 (FP64 Jacobian and inner solve).

    An interval is one backward-Euler step of dt; when Newton does not
    reach the FP64 relative residual 1e-8 (within ``attempt_max_it``
    iterations; the step test is off, so no step ends on a small update
    above the tolerance) the interval is redone as
    four steps of dt/4, recursively up to ``max_cuts`` levels: the cut of the
    reference's time integrator (dt * 0.25 on a failed step,
    src/tdyti.c:140-150).  Every backward-Euler step of the mixed run is
    checked against the FP64 oracle: ||F(U_k+1)|| / ||F(U_k)|| with the
    oracle's residual at that step's dt (threaded oracle)."""
    import torch

    import tdycore_gb300 as T
    from tdycore_gb300.workloads import infiltration_prisms
    from oracle import Oracle

    T.options_clear()
    t0 = time.perf_counter()
    t, U0, top, src, info = infiltration_prisms(ntri, nlayers, rotation=rotation)
    t.setup()
    t.set_source_sink_values(src, cells=top)
    setup_s = time.perf_counter() - t0
    nc, nnz = t.ncells, int(t.nnz)
    log(f"config 3: {nc} cells, nnz {nnz}, setup {setup_s:.1f} s")
    o = Oracle(t.setup_view())
    dev = torch.device("cuda")
    # warm-up: spmv autotune and the inner-solve graphs of both arithmetic modes
    for fp32 in (True, False):
        w = torch.tensor(U0, dtype=torch.float64, device=dev)
        t.backward_euler_step_device(w, dt / 4 ** max_cuts, fp32=fp32, precond=precond, max_it=attempt_max_it,
                                     stol=0.0)
    del w

    def advance(d, h, level, fp32, recs, check):
        """One step of h, or four of h/4 (recursively) when it fails; appends
        a record per backward-Euler step attempted; False if a step at the
        deepest level fails."""
        save = d.clone()
        torch.cuda.synchronize()
        ts = time.perf_counter()
        st, its, rel = t.backward_euler_step_device(d, h, fp32=fp32, precond=precond, max_it=attempt_max_it,
                                                    stol=0.0)
        torch.cuda.synchronize()
        ok = st["converged"] == 1
        rec = {"dt": h, "level": level, "converged": st["converged"] == 1,
               "ended_by_step_test": st["step_converged"] == 1, "newton": int(its[0]),
               "linear": st["linear_iterations"], "rel_residual_device": float(rel[0]),
               "s": time.perf_counter() - ts, "eval_s": st["eval_s"], "precond_s": st["precond_s"],
               "krylov_s": st["krylov_s"]}
        if ok and check:
            un, u1 = save.cpu().numpy(), d.cpu().numpy()
            o.snes_presolve(un, h)
            f0 = np.linalg.norm(o.snes_function_parallel(un, oracle_threads))
            rec["oracle_rel_residual"] = float(np.linalg.norm(o.snes_function_parallel(u1, oracle_threads)) / f0)
        recs.append(rec)
        if ok:
            return True
        d.copy_(save)
        if level == max_cuts:
            return False
        for _ in range(4):
            if not advance(d, h / 4, level + 1, fp32, recs, check):
                return False
        return True

    arms = {}
    for name, fp32 in (("mixed", True), ("fp64", False)):
        d = torch.tensor(U0, dtype=torch.float64, device=dev)
        per_interval, total, completed = [], 0.0, 0
        phases = {"eval_s": 0.0, "precond_s": 0.0, "krylov_s": 0.0}
        for k in range(steps):
            recs = []
            ok = advance(d, dt, 0, fp32, recs, check=fp32)
            solve_s = sum(r["s"] for r in recs)  # device solves only (oracle checks excluded)
            total += solve_s
            for key in phases:
                phases[key] += sum(r[key] for r in recs)
            done = [r for r in recs if r["converged"] or r["ended_by_step_test"]]
            row = {"interval": k + 1, "ok": ok, "be_steps": len(done), "failed_attempts": len(recs) - len(done),
                   "deepest_cut": max(r["level"] for r in recs), "newton": sum(r["newton"] for r in recs),
                   "linear": sum(r["linear"] for r in recs), "solve_s": solve_s}
            if fp32:
                chk = [r["oracle_rel_residual"] for r in done if "oracle_rel_residual" in r]
                row["oracle_rel_residual_max"] = max(chk) if chk else None
                row["ended_by_step_test"] = sum(r["ended_by_step_test"] for r in done)
            per_interval.append(row)
            log(f"config 3 {name} interval {k + 1}: {row}")
            if not ok:
                break
            completed += 1
        phases["other_s"] = total - sum(phases.values())  # line-search and convergence bookkeeping, host work
        arms[name] = {"intervals_completed": completed, "solve_s_total": total, "phases_s": phases,
                      "per_interval": per_interval, "U": d.cpu().numpy()}
    m, f = arms["mixed"], arms["fp64"]
    U = m.pop("U")
    U64 = f.pop("U")
    t.destroy()
    T.options_clear()
    checked = [r["oracle_rel_residual_max"] for r in m["per_interval"] if r.get("oracle_rel_residual_max") is not None]
    return {
        "workload": info["workload"], "ncells": nc, "nnz_jacobian": nnz,
        "rotation": info["rotation"], "van_genuchten": info["van_genuchten"], "preconditioner": precond,
        "initial_pressure_pa": info["initial_pressure_pa"], "depth_m": info["depth_m"],
        "top_flux_m_per_s": info["top_flux_m_per_s"], "dt_s": dt, "intervals": steps, "setup_s": setup_s,
        "cut_policy": f"a failed step is redone as 4 steps of dt/4, up to {max_cuts} levels (src/tdyti.c:140-150); "
                      f"an attempt fails after {attempt_max_it} Newton iterations",
        "mixed": m, "fp64": f,
        "all_intervals_completed_mixed": m["intervals_completed"] == steps,
        "max_oracle_rel_residual": max(checked) if checked else None,
        "speedup_mixed_vs_fp64": (f["solve_s_total"] / m["solve_s_total"]) if m["solve_s_total"] > 0 else None,
        "final_max_rel_diff_mixed_vs_fp64": float(np.max(np.abs(U - U64) / np.abs(U64))),
        "pressure_range_pa_final": [float(U.min()), float(U.max())],
        "note": "mixed = FP64 residual with FP32 Jacobian and inner solve; fp64 = FP64 Jacobian and inner solve, "
                "its own trajectory from the same start; oracle_rel_residual = ||F(U_k+1)|| / ||F(U_k)|| per "
                "backward-Euler step of the mixed run from the FP64 CPU oracle (threaded); phases_s = device time "
                "on the solve's stream in F+J evaluations (line-search trials included), Jacobian copies and "
                "preconditioner set-ups, and BiCGStab iterations; the precision of the inner solve changes only "
                "the last two",
    }


def prisms_eval_full_size(ntri=200_000, nlayers=40, reps=10, dt=3600.0):
    """Config 3 at its full size and tensor field (Delaunay prisms, per-cell
    K with a uniform random 3-D rotation): one mixed-form evaluation (FP64
    residual, Jacobian rounded to FP32 for the inner solve) against the FP64
    oracle, and the device F+J time, at a state with saturated and
    unsaturated cells."""
    import torch

    import tdycore_gb300 as T
    from tdycore_gb300.workloads import infiltration_prisms
    from oracle import Oracle

    T.options_clear()
    t0 = time.perf_counter()
    t, U0, top, src, info = infiltration_prisms(ntri, nlayers, rotation="full")
    t.setup()
    t.set_source_sink_values(src, cells=top)
    setup_s = time.perf_counter() - t0
    nc, nnz = t.ncells, int(t.nnz)
    rng = np.random.default_rng(5)
    U = U0 + 2.0e4 + rng.normal(0.0, 2.0e3, nc)
    Uprev = U + rng.normal(0.0, 50.0, nc)
    dev = torch.device("cuda")
    dU = torch.tensor(U, dtype=torch.float64, device=dev)
    dUp = torch.tensor(Uprev, dtype=torch.float64, device=dev)
    dR = torch.empty(nc, dtype=torch.float64, device=dev)
    dJ = torch.empty(nnz, dtype=torch.float64, device=dev)
    st = torch.cuda.Stream(device=dev)  # the launches and the events on one (non-null) stream
    t.set_dtime(dt)
    t.presolve_device(dUp, stream=st.cuda_stream)
    for _ in range(3):
        t.snes_function_jacobian_device(dU, dR, dJ, stream=st.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        t.snes_function_jacobian_device(dU, dR, dJ, stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    R, J, J32 = dR.cpu().numpy(), dJ.cpu().numpy(), dJ.float().cpu().numpy().astype(np.float64)
    o = Oracle(t.setup_view())
    o.snes_presolve(Uprev, dt)
    Rr, Rm = o.snes_function(U, with_mag=True)
    Jr, Jm = o.snes_jacobian(U, with_mag=True)
    tiny = np.finfo(float).tiny
    nzj = np.abs(Jr) > 0
    t.destroy()
    T.options_clear()
    return {"workload": info["workload"], "ncells": nc, "nnz_jacobian": nnz, "rotation": "full",
            "setup_s": setup_s, "fj_ms": ms, "fj_cells_per_s": nc / (ms * 1e-3),
            "R_err_over_scale": float(np.max(np.abs(R - Rr) / np.maximum(Rm, tiny))),
            "J_fp64_err_over_scale": float(np.max(np.abs(J - Jr) / np.maximum(Jm, tiny))),
            "J_fp32_err_over_scale": float(np.max(np.abs(J32 - Jr) / np.maximum(Jm, tiny))),
            "J_fp32_max_rel_err": float(np.max(np.abs(J32[nzj] - Jr[nzj]) / np.abs(Jr[nzj]))),
            "note": "state: uniform Pref plus N(0, 2 kPa) (saturated and unsaturated cells), previous state "
                    "N(0, 50 Pa) from it; errors in units of the oracle's per-entry error scale"}


def profile_prisms(ntri, evaluations, dt=3600.0):
    """Only the device F+J of the prism workload (3-D rotated K, a state with
    saturated and unsaturated cells), ``evaluations`` times, for profilers."""
    import torch

    import tdycore_gb300 as T
    from tdycore_gb300.workloads import infiltration_prisms

    T.options_clear()
    t, U0, top, src, info = infiltration_prisms(ntri, 40, rotation="full")
    t.setup()
    t.set_source_sink_values(src, cells=top)
    nc, nnz = t.ncells, int(t.nnz)
    dev = torch.device("cuda")
    st = torch.cuda.Stream(device=dev)
    U = U0 + 2.0e4 + np.random.default_rng(5).normal(0.0, 2.0e3, nc)
    dU = torch.tensor(U, dtype=torch.float64, device=dev)
    dUp = dU + 10.0
    dR = torch.empty(nc, dtype=torch.float64, device=dev)
    dJ = torch.empty(nnz, dtype=torch.float64, device=dev)
    t.set_dtime(dt)
    t.presolve_device(dUp, stream=st.cuda_stream)
    for _ in range(evaluations):
        t.snes_function_jacobian_device(dU, dR, dJ, stream=st.cuda_stream)
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": info["workload"], "ncells": nc, "nnz": nnz, "evaluations": evaluations}))


def profile_batch(ninst, steps=2, dt=3600.0):
    """Only the batched device Newton of ``ninst`` config-4 instances
    (``steps`` backward-Euler steps from the same start, FP32 inner solves,
    autotuned schedules), for profilers."""
    import torch

    import tdycore_gb300 as T
    from tdycore_gb300.workloads import batched_columns

    T.options_clear()
    T.options_insert("-tdy_mpfao_setup_on_device")
    tb, U0, info = batched_columns(ninst)
    tb.setup()
    out = []
    for _ in range(steps):
        d = torch.tensor(U0, dtype=torch.float64, device="cuda")
        st, its, rel = tb.backward_euler_step_device(d, dt)
        torch.cuda.synchronize()
        out.append({k: st[k] for k in ("converged", "newton_iterations", "linear_iterations", "block_instances",
                                        "eval_schedule")})
    tb.destroy()
    print(json.dumps({"profile_batch": info["workload"], "ncells": int(sum(info["instance_cells"])), "runs": out}))


def serving_config5(nreq=160, rate=80.0, slots=8, cohort=32):
    """Config 5: Poisson arrivals of column/subdomain requests (5 % of them
    64 x 64 x 50 cells), 24 hourly backward-Euler steps each with top-flux
    forcing, state resident on the device, admission by HBM footprint against
    150 GB; continuous batching (``slots`` workers, each serving a cohort of up
    to ``cohort`` waiting requests as one batched handle, FP32 inner solves)
    next to plain FP64 one-at-a-time serving of the same requests.  Eight
    workers with cohorts of up to 32 measured best in throughput and latency
    (fewer host threads make fewer concurrent driver calls): 564 solves/s,
    p99 5.2 s, against 451-540 solves/s with 16 or 32 workers."""
    from tdycore_gb300 import serving as S

    out = {}
    for name, kw in (("continuous_fp32", {"slots": slots, "fp32": True, "cohort": cohort}),
                     ("one_at_a_time_fp64", {"slots": 1, "fp32": False, "cohort": 1})):
        reqs = S.make_requests(nreq, rate_per_s=rate, nsteps=24, large_fraction=0.05, seed=0)
        srv = S.Server(hbm_budget_bytes=150e9, **kw)
        t0 = time.perf_counter()
        done = srv.run(reqs)
        wall = time.perf_counter() - t0
        out[name] = S.summary(done, wall)
        out[name]["peak_workers_in_flight"] = srv.peak_running
        out[name]["cohorts"] = {"count": len(srv.cohorts), "mean_size": float(np.mean(srv.cohorts)),
                                "max_size": int(max(srv.cohorts))}
        out[name]["peak_hbm_reserved_GB"] = srv.peak_in_use / 1e9
        log(f"config 5 {name}: {out[name]}")
    out["requests"] = nreq
    out["arrival_rate_per_s"] = rate
    out["large_requests"] = int(sum((r.nx, r.ny, r.nz) == (64, 64, 50)
                                    for r in S.make_requests(nreq, rate, 24, 0.05, 0)))
    c, o = out["continuous_fp32"], out["one_at_a_time_fp64"]
    out["solves_per_s_ratio"] = c["solves_per_s"] / o["solves_per_s"]
    return out


def cpu_baseline(o, U, budget_s=12.0, threads=None):
    ncells = U.size
    """Oracle F+J (reference loop order, colour-parallel) on the host cores."""
    cores = threads or len(os.sched_getaffinity(0))
    log(f"CPU baseline on {cores} threads")
    o.snes_function_jacobian_parallel(U, cores)  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        o.snes_function_jacobian_parallel(U, cores)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 50:
            break
    return ncells * n / el, cores, n, el


def run_reference(args, rank):
    if rank != 0:
        return
    t, U, Uprev, info = build_workload(host_only=True, grid=args.grid)
    view = t.setup_view()
    from oracle import Oracle

    cores = len(os.sched_getaffinity(0))
    o = Oracle(view)
    o.snes_presolve(Uprev, DT)
    for _ in range(max(1, min(args.warmup, 3))):
        o.snes_function_jacobian_parallel(U, cores)
    steps = max(1, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.snes_function_jacobian_parallel(U, cores)
    el = time.perf_counter() - t0
    value = view["ncells"] * steps / el
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(info, view["ncells"], int(view["nnz"]), args.gpus),
        "jacobian_arithmetic": "FP64",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{steps} full F+J evaluations of the {view['ncells']}-cell workload"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C restatement of the reference loops (oracle/); the reference needs PETSc+MPI, absent here",
    }
    print(json.dumps(out), flush=True)


def run_gpu(args, rank, world, local_rank):
    import torch

    import tdycore_gb300 as T

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    t, U, Uprev, info = build_workload(grid=args.grid, jacobian_arithmetic=args.jacobian_arithmetic)
    view = t.setup_view()
    nc, nnz = t.ncells, t.nnz
    t.set_dtime(DT)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    dU = torch.tensor(U, dtype=torch.float64, device=dev)
    dUp = torch.tensor(Uprev, dtype=torch.float64, device=dev)
    dR = torch.empty(nc, dtype=torch.float64, device=dev)
    dJ = torch.empty(nnz, dtype=torch.float64, device=dev)
    sp = stream.cuda_stream
    t.presolve_device(dUp, stream=sp)
    for _ in range(args.warmup):
        t.snes_function_jacobian_device(dU, dR, dJ, stream=sp)
    torch.cuda.synchronize(dev)

    # device-resident throughput
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            t.snes_function_jacobian_device(dU, dR, dJ, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if not args.profile and args.steps * 0.001 < 1.0:  # keep ~1 s of load for the clock record
            tt = time.perf_counter()
            while time.perf_counter() - tt < 1.0:
                t.snes_function_jacobian_device(dU, dR, dJ, stream=sp)
                torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    if dist:
        tms = torch.tensor([ms], device=dev)
        dist.all_reduce(tms, op=dist.ReduceOp.MAX)
        ms = float(tms.item())
    ms_per_step = ms / args.steps
    value = world * nc * args.steps / (ms * 1e-3)

    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": info["workload"], "ncells": nc, "ms_per_step": ms / args.steps}))
        return
    # per-kernel durations (events between launches)
    t.set_timers(True)
    kt_steps = min(args.steps, 50)
    for _ in range(kt_steps):
        t.snes_function_jacobian_device(dU, dR, dJ, stream=sp)
    timers = t.timers()
    t.set_timers(False)
    kernel_ms = {k: v[0] / max(v[1], 1) for k, v in timers.items()}
    eval_ms = sum(kernel_ms.values())

    # end to end through the host-pointer C-ABI (pinned buffers)
    Uh = torch.tensor(U, dtype=torch.float64).pin_memory()
    Rh = torch.empty(nc, dtype=torch.float64).pin_memory()
    Jh = torch.empty(nnz, dtype=torch.float64).pin_memory()
    Un, Rn, Jn = Uh.numpy(), Rh.numpy(), Jh.numpy()
    e2e_steps = max(3, min(args.steps, 30))

    def end_to_end(tt_):
        tt_.presolve(Uprev)
        for _ in range(2):
            tt_.snes_function_jacobian(Un, Rn, Jn)
        if dist:
            dist.barrier()
        t_0 = time.perf_counter()
        for _ in range(e2e_steps):
            tt_.snes_function_jacobian(Un, Rn, Jn)
        el = time.perf_counter() - t_0
        if dist:
            te = torch.tensor([el], device=dev)
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
            el = float(te.item())
        return world * nc * e2e_steps / el

    e2e_value = end_to_end(t)
    e2e_out = (Rn.copy(), Jn.copy())  # the host-pointer call's last R and J (slab pipeline)

    # the same device loop and end-to-end call with FP64 Jacobian products
    R_main, J_main = dR.cpu().numpy(), dJ.cpu().numpy()
    e2e_bits_equal = bool(np.array_equal(e2e_out[0], R_main) and np.array_equal(e2e_out[1], J_main))
    alt = None
    if args.jacobian_arithmetic != "FP64":
        t.destroy()
        del t
        t2, _, _, info2 = build_workload(grid=args.grid, jacobian_arithmetic="FP64",
                                         extra_options="-tdy_mpfao_setup_on_device")
        t2.set_dtime(DT)
        t2.presolve_device(dUp, stream=sp)
        for _ in range(max(3, args.warmup)):
            t2.snes_function_jacobian_device(dU, dR, dJ, stream=sp)
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        e0.record(stream)
        for _ in range(args.steps):
            t2.snes_function_jacobian_device(dU, dR, dJ, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms2 = e0.elapsed_time(e1)
        if dist:
            tms = torch.tensor([ms2], device=dev)
            dist.all_reduce(tms, op=dist.ReduceOp.MAX)
            ms2 = float(tms.item())
        alt = {"jacobian_arithmetic": "FP64", "setup_s": info2["setup_s"],
               "value": world * nc * args.steps / (ms2 * 1e-3),
               "ms_per_step": ms2 / args.steps, "R": dR.cpu().numpy(), "J": dJ.cpu().numpy()}
        alt["e2e"] = end_to_end(t2)
        t2.presolve_device(dUp, stream=sp)  # the device loop's accumulation state for the FP64 parity check
        launches = t2.launches_per_evaluation()
        t2.destroy()
    else:
        launches = t.launches_per_evaluation()

    if rank == 0:
        hbm_peak, peak_kind = peaks()
        try:
            fp64_peak = T.device_fp64_tflops()
        except Exception:
            fp64_peak = None
        vb = vertex_kernel_bytes(view)
        vk_ms = kernel_ms.get("vertex_kernel", float("nan"))
        achieved = vb / (vk_ms * 1e-3) / 1e9
        balg = algorithmic_bytes(view)
        traffic = None
        tf = ROOT / "profiles" / "vertex_kernel_traffic.json"
        if tf.exists():
            try:
                traffic = json.loads(tf.read_text()).get("bytes_per_launch_full_workload")
            except Exception:
                traffic = None
        o = make_oracle(view, Uprev)
        parity = {}
        (parity["R_err_over_scale"], parity[f"J_err_over_scale_{args.jacobian_arithmetic.lower()}"],
         parity["R_rel_l2"]) = parity_full_size(o, U, R_main, J_main)
        if alt is not None:
            rr, jj, rl2 = parity_full_size(o, U, alt["R"], alt["J"])
            parity["R_err_over_scale_fp64_device_trans"] = rr
            parity["J_err_over_scale_fp64_device_trans"] = jj
            parity["R_rel_l2_fp64_device_trans"] = rl2
        parity["bars"] = {"R": 1e-12, "J": 1e-10, "R_rel_l2": 1e-12}
        parity["state"] = "hydrostatic plus N(0, 5 kPa) noise (far from equilibrium); previous state N(0, 200 Pa) off"
        cpu_v, cores, n_cpu, cpu_s = cpu_baseline(o, U, budget_s=args.cpu_budget)
        del o
        cfg1 = {}
        for start in ("hydrostatic", "dry"):
            try:
                cfg1[start] = newton_config1(start)
            except Exception as e:  # reported, never fatal to the headline line
                cfg1[start] = {"error": repr(e)}
        cfg5 = None
        if args.serve_requests > 0:
            try:
                cfg5 = serving_config5(args.serve_requests)
            except Exception as e:
                cfg5 = {"error": repr(e)}
        cfg3 = None
        if args.prisms_triangles > 0:
            try:
                cfg3 = prisms_config3(args.prisms_triangles, dt=args.prisms_dt, precond=args.prisms_precond,
                                      steps=args.prisms_steps)
            except Exception as e:
                cfg3 = {"error": repr(e)}
        if args.prisms_eval_triangles > 0:
            try:
                ev = prisms_eval_full_size(args.prisms_eval_triangles)
            except Exception as e:
                ev = {"error": repr(e)}
            cfg3 = dict(cfg3 or {}, mixed_form_evaluation=ev)
        cfg4 = None
        if args.batch_instances > 0:
            try:
                cfg4 = batched_config4(args.batch_instances)
            except Exception as e:
                cfg4 = {"error": repr(e)}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(info, nc, nnz, world),
            "jacobian_arithmetic": args.jacobian_arithmetic,
            "roofline": {"bound": "hbm", "kernel": "vertex_kernel", "achieved": achieved, "peak": hbm_peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": vb,
                         "algorithmic_bytes_formula": "8 * (sum_v R_v C_v + sum_v R_v + Nc): Trans, gravity "
                                                      "term per row, cell pressures",
                         "avg_launch_ms": vk_ms,
                         "binding_roof": "FP64 pipe (see fp64.pipe_active_ncu)"},
            "roofline_evaluation": {"algorithmic_bytes": balg, "GBps": balg / (ms_per_step * 1e-3) / 1e9,
                                    "frac_hbm": balg / (ms_per_step * 1e-3) / 1e9 / hbm_peak,
                                    "bytes_per_cell": balg / nc},
            "fp64": {"peak_tflops_probe": fp64_peak, "pipe_active_ncu": fp64_pipe_from_profile(kernel_ms)},
            "kernel_ms": kernel_ms,
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n_cpu} full F+J evaluations ({cpu_s:.1f} s) of the same workload"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * nc,
                    "d2h_bytes_per_step": 8 * (nc + nnz), "steps": e2e_steps,
                    "R_J_equal_device_path": e2e_bits_equal},
            "gpu_launches": args.steps * launches,
            "parity_full_size": parity,
            "config1_newton": cfg1,
            "config3_prisms_mixed_precision": cfg3,
            "config4_batched": cfg4,
            "config5_serving": cfg5,
            "setup_s": {"trans_on_host": info["setup_s"],
                        "trans_on_device": alt["setup_s"] if alt is not None else None,
                        "note": "TDySetup wall time (mesh, materials, interaction regions, layouts, upload); "
                                "-tdy_mpfao_setup_on_device builds the interior vertices' Trans on the GPU"},
            "clocks": clk.summary(),
        }
        if alt is not None:
            out["fp64_jacobian"] = {"value": alt["value"], "unit": UNIT, "ms_per_step": alt["ms_per_step"],
                                    "e2e": {"value": alt["e2e"], "unit": UNIT, "h2d_bytes_per_step": 8 * nc,
                                            "d2h_bytes_per_step": 8 * (nc + nnz), "steps": e2e_steps},
                                    "note": "strict FP64: the same device loop and end-to-end call with "
                                            "-tdy_jacobian_arithmetic FP64 (and Trans built on the device)"}
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--grid", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="smaller grid with the same extents per cell (profiling captures)")
    ap.add_argument("--jacobian-arithmetic", default="DOUBLE_FLOAT", choices=["DOUBLE_FLOAT", "FP64"],
                    help="arithmetic of the Jacobian products at interior hexahedral vertices")
    ap.add_argument("--serve-requests", type=int, default=160,
                    help="requests of the serving measurement (0 skips it)")
    ap.add_argument("--prisms-triangles", type=int, default=200000,
                    help="surface triangles of the prism infiltration measurement (0 skips it; 200000 x 40 layers "
                         "is the configuration's 8 M cells)")
    ap.add_argument("--prisms-dt", type=float, default=1.0,
                    help="time step of the prism infiltration measurement (s)")
    ap.add_argument("--prisms-precond", default="clusters", choices=["lines", "clusters"],
                    help="inner-solve preconditioner of the prism infiltration measurement")
    ap.add_argument("--prisms-steps", type=int, default=20,
                    help="backward-Euler steps of the prism infiltration measurement")
    ap.add_argument("--prisms-eval-triangles", type=int, default=200000,
                    help="surface triangles of the mixed-form F+J evaluation on prisms with 3-D rotated K "
                         "(200000 is the full configuration; 0 skips it)")
    ap.add_argument("--batch-instances", type=int, default=4096,
                    help="instances of the batched-solve measurement (0 skips it)")
    ap.add_argument("--profile-prisms", type=int, default=0, metavar="NTRI",
                    help="only --steps device F+J evaluations of the prism workload with NTRI surface "
                         "triangles and 40 layers (for ncu)")
    ap.add_argument("--profile-batch", type=int, default=0, metavar="NINST",
                    help="only the batched device Newton of NINST config-4 instances (for ncu)")
    ap.add_argument("--profile", action="store_true",
                    help="time the device loop only (no timers, e2e, CPU or clock-fill loops), for ncu")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.profile_prisms > 0:
        profile_prisms(args.profile_prisms, args.steps)
    elif args.profile_batch > 0:
        profile_batch(args.profile_batch, max(1, min(args.steps, 4)))
    elif args.impl == "reference":
        run_reference(args, rank)
    else:
        run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
