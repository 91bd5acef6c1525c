"""Continuous-batching request server over the device Newton solver.

Each request is an independent Richards problem: a hexahedral soil column or
small 3-D subdomain with its own parameters, advanced ``nsteps`` hourly
backward-Euler steps with a top-flux forcing per step (a source in the top
layer, rho * q * A kg/s per top cell).  Its state stays on the device for
the whole request.

Serving is continuous: a request that arrives while others are on the GPU is
admitted as soon as a slot and enough of the HBM budget are free, and its
steps overlap on the device with those of the requests already running.
Requests are admitted in cohorts: when a slot frees up, the requests that
have arrived and wait (up to ``cohort`` of them, consecutive in arrival
order and of one size class) become one batched handle, each request an
instance, driven by one worker thread (the C-ABI calls release the
interpreter lock).  A cohort's Newton iterations evaluate and solve only its
instances still iterating (one CTA per instance), and a request that fails
a step is retired from its cohort.  An instance gets the same bits alone and
in any batch (every schedule gives the same bits, reductions are chunked per
instance), so a request's result is the same alone and in any mix.

No reference counterpart: TDycore runs one problem per process through
PETSc.
"""
from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import NEUMANN_BC, WATER_DENSITY_CONSTANT, create_richards_mpfao, options_clear, options_insert
from .workloads import GRAVITY, PREF, layered_z, structured_surface

RHO = 998.0  # constant water density of the EOS used here (kg/m^3)


@dataclass
class Request:
    rid: int
    arrival_s: float
    nx: int
    ny: int
    nz: int
    dz: float
    k: float          # isotropic permeability (m^2)
    porosity: float
    alpha: float      # van Genuchten alpha (1/Pa)
    m: float          # van Genuchten / Mualem m
    forcing: np.ndarray  # top flux per step (m/s, positive into the domain)
    sr: float = 0.15
    cell: float = 1.0
    # filled by the server
    admitted_s: float = float("nan")
    finished_s: float = float("nan")
    U_final: np.ndarray | None = field(default=None, repr=False)
    newton_its: list = field(default_factory=list)
    rel_residual: list = field(default_factory=list)
    converged_steps: int = 0
    step_test_steps: int = 0  # steps ended by the step test above the tolerance
    setup_s: float = float("nan")  # building the request's handle (host mesh and layouts, Trans on the device)
    error: str | None = None

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def latency_s(self) -> float:
        return self.finished_s - self.arrival_s


def footprint_bytes(ncells: int) -> int:
    """Device bytes one request holds: state, per-vertex partials, Jacobian
    in FP64 and FP32, Krylov vectors and mesh arrays (about 2 KB per cell),
    plus a fixed 16 MB."""
    return 2048 * ncells + (16 << 20)


def build(req: Request):
    """Handle and initial state of a request: hydrostatic with the water table
    at 60 % of the height (plus 10 Pa of seeded noise, which keeps vertical
    faces off exact upwinding ties), no-flow boundaries, forcing as a source."""
    xy, quads = structured_surface(req.nx, req.ny, req.cell * req.nx, req.cell * req.ny)
    depth = req.dz * req.nz
    z = layered_z(xy.shape[0], req.nz, depth)
    t = create_richards_mpfao()
    t.set_extruded_meshes([(xy, quads, z)])
    t.set_from_options()
    n = req.ncells
    K = np.zeros((n, 9))
    K[:, 0] = K[:, 4] = K[:, 8] = req.k
    t.set_permeability_values(K)
    t.set_porosity_values(np.full(n, req.porosity))
    t.set_vangenuchten_values(np.full(n, req.m), np.full(n, req.alpha))
    t.set_mualem_values(np.full(n, req.m))
    t.set_constant_residual_saturation(req.sr)
    t.set_water_density_type(WATER_DENSITY_CONSTANT)
    t.set_boundary_pressure_type_function(lambda x, y, zz: np.full(np.shape(x), NEUMANN_BC))
    zc = (np.arange(req.nz) + 0.5) * req.dz
    p = PREF + RHO * GRAVITY * (0.6 * depth - zc)
    U0 = np.repeat(p, req.nx * req.ny) + np.random.default_rng(1000 + req.rid).normal(0.0, 10.0, n)
    top = np.arange((req.nz - 1) * req.nx * req.ny, n, dtype=np.int32)
    return t, U0, top


_opts_lock = threading.Lock()
_opts_cleared = False


def options_clear_once():
    """Requests read one option: their interaction-region transmissibilities
    are built on the device (-tdy_mpfao_setup_on_device), which shortens
    admission.  The database is set once per process, so a caller's
    leftovers do not leak into request handles (TDySetFromOptions only reads
    it, from any thread)."""
    global _opts_cleared
    with _opts_lock:
        if not _opts_cleared:
            options_clear()
            options_insert("-tdy_mpfao_setup_on_device")
            _opts_cleared = True


def run_request(req: Request, fp32: bool = True, dt: float = 3600.0, rtol: float = 1e-8):
    """All steps of one request on the calling thread (its own handle and
    stream); fills the request's results."""
    import torch

    options_clear_once()
    ts = time.perf_counter()
    t, U0, top = build(req)
    t.setup()
    req.setup_s = time.perf_counter() - ts
    try:
        dU = torch.tensor(U0, dtype=torch.float64, device="cuda")
        torch.cuda.current_stream().synchronize()
        area = req.cell * req.cell
        for k, q in enumerate(req.forcing):
            t.set_source_sink_values(np.full(top.size, RHO * q * area), cells=top)
            stats, its, rel = t.backward_euler_step_device(dU, dt, rtol=rtol, fp32=fp32)
            req.newton_its.append(int(its[0]))
            req.rel_residual.append(float(rel[0]))
            if stats["step_converged"] == 1:
                # Newton stopped on a negligible step above the tolerance (as
                # PETSc's step test does): the request goes on, but the step
                # is not counted as a solve at the tolerance
                req.step_test_steps += 1
                continue
            if stats["converged"] != 1:
                # the request ends here: later steps from an unconverged state
                # would mean nothing to the caller
                req.error = f"step {k + 1} did not converge (relative residual {rel[0]:.1e})"
                break
            req.converged_steps += 1
        req.U_final = dU.cpu().numpy()
    finally:
        t.destroy()


LARGE_CELLS = 100_000  # requests of at least this many cells form cohorts of one


def size_class(r: Request) -> int:
    return 1 if r.ncells >= LARGE_CELLS else 0


def build_cohort(reqs):
    """One batched handle for ``reqs`` (each request's mesh a block, with the
    properties, boundary conditions and initial state ``build`` gives it
    alone); returns (handle, U0, top cells per request)."""
    blocks, K, poro, m, alpha, sr, U0, tops = [], [], [], [], [], [], [], []
    off = 0
    for r in reqs:
        xy, quads = structured_surface(r.nx, r.ny, r.cell * r.nx, r.cell * r.ny)
        depth = r.dz * r.nz
        blocks.append((xy, quads, layered_z(xy.shape[0], r.nz, depth)))
        n = r.ncells
        k = np.zeros((n, 9))
        k[:, 0] = k[:, 4] = k[:, 8] = r.k
        K.append(k)
        poro.append(np.full(n, r.porosity))
        m.append(np.full(n, r.m))
        alpha.append(np.full(n, r.alpha))
        sr.append(np.full(n, r.sr))
        zc = (np.arange(r.nz) + 0.5) * r.dz
        p = PREF + RHO * GRAVITY * (0.6 * depth - zc)
        U0.append(np.repeat(p, r.nx * r.ny) + np.random.default_rng(1000 + r.rid).normal(0.0, 10.0, n))
        tops.append(off + np.arange((r.nz - 1) * r.nx * r.ny, n, dtype=np.int32))
        off += n
    t = create_richards_mpfao()
    t.set_extruded_meshes(blocks)
    t.set_from_options()
    t.set_permeability_values(np.concatenate(K))
    t.set_porosity_values(np.concatenate(poro))
    mm = np.concatenate(m)
    t.set_vangenuchten_values(mm, np.concatenate(alpha))
    t.set_mualem_values(mm)
    t.set_residual_saturation_values(np.concatenate(sr))
    t.set_water_density_type(WATER_DENSITY_CONSTANT)
    t.set_boundary_pressure_type_function(lambda x, y, zz: np.full(np.shape(x), NEUMANN_BC))
    return t, np.concatenate(U0), tops


def run_cohort(reqs, fp32: bool = True, dt: float = 3600.0, rtol: float = 1e-8, finished=None):
    """All steps of the requests of one cohort on the calling thread: one
    batched handle, each request an instance; a request that does not
    converge a step is retired (its error recorded) and the others go on.
    ``finished(r)`` is called as each request completes."""
    import torch

    from . import INSTANCE_CONVERGED, INSTANCE_STEP_TEST

    options_clear_once()
    ts = time.perf_counter()
    t, U0, tops = build_cohort(reqs)
    t.setup()
    setup_s = time.perf_counter() - ts
    for r in reqs:
        r.setup_s = setup_s
    top_all = np.concatenate(tops)
    area = np.concatenate([np.full(tp.size, r.cell * r.cell) for r, tp in zip(reqs, tops)])
    try:
        dU = torch.tensor(U0, dtype=torch.float64, device="cuda")
        torch.cuda.current_stream().synchronize()
        done = [False] * len(reqs)
        for k in range(max(len(r.forcing) for r in reqs)):
            active = np.array([not done[i] and k < len(r.forcing) for i, r in enumerate(reqs)], dtype=np.int32)
            if not active.any():
                break
            q = np.concatenate([np.full(tp.size, r.forcing[k] if active[i] else 0.0)
                                for i, (r, tp) in enumerate(zip(reqs, tops))])
            t.set_source_sink_values(RHO * q * area, cells=top_all)
            t.set_active_instances(active)
            stats, its, rel = t.backward_euler_step_device(dU, dt, rtol=rtol, fp32=fp32)
            status = t.instance_status()
            for i, r in enumerate(reqs):
                if not active[i]:
                    continue
                r.newton_its.append(int(its[i]))
                r.rel_residual.append(float(rel[i]))
                if status[i] == INSTANCE_CONVERGED:
                    r.converged_steps += 1
                elif status[i] == INSTANCE_STEP_TEST:
                    r.step_test_steps += 1
                else:
                    r.error = f"step {k + 1} did not converge (relative residual {rel[i]:.1e})"
                if r.error is not None or k + 1 == len(r.forcing):
                    done[i] = True
                    if r.error is None:
                        c0, c1 = (int(tops[i][0]) - (r.nz - 1) * r.nx * r.ny, int(tops[i][-1]) + 1)
                        r.U_final = dU[c0:c1].cpu().numpy()
                    if finished:
                        finished(r)
        Uh = dU.cpu().numpy()
        off = np.concatenate([[0], np.cumsum([r.ncells for r in reqs])])
        for i, r in enumerate(reqs):
            if r.U_final is None:
                r.U_final = Uh[off[i]:off[i + 1]].copy()
    finally:
        t.destroy()


class Server:
    """Admits requests in arrival order as slots and HBM budget allow and runs
    them concurrently (``slots`` worker threads), ``cohort`` requests of one
    size class at most per worker (``cohort=1``: one handle per request)."""

    def __init__(self, slots: int = 8, hbm_budget_bytes: float = 150e9, fp32: bool = True, dt: float = 3600.0,
                 runner=None, footprint=footprint_bytes, clock=time.perf_counter, cohort: int = 32):
        self.slots, self.budget, self.fp32, self.dt = slots, float(hbm_budget_bytes), fp32, dt
        self.cohort = max(1, cohort)
        if runner is None:
            if self.cohort == 1:
                runner = lambda reqs, finished: run_request(reqs[0], fp32=self.fp32, dt=self.dt)  # noqa: E731
            else:
                runner = lambda reqs, finished: run_cohort(reqs, fp32=self.fp32, dt=self.dt,  # noqa: E731
                                                           finished=finished)
        self.runner = runner
        self.footprint = footprint
        self.clock = clock
        self.peak_in_use = 0.0
        self.peak_running = 0
        self.cohorts = []  # sizes of the cohorts formed

    def run(self, requests):
        """Serves ``requests`` (their arrival_s relative to the start) and
        returns them with admission/finish times and results."""
        reqs = sorted(requests, key=lambda r: r.arrival_s)
        for r in reqs:
            if self.footprint(r.ncells) > self.budget:
                raise ValueError(f"request {r.rid} needs more than the whole HBM budget")
        lock = threading.Condition()
        in_use, running = [0.0], [0]
        start = self.clock()

        def finished(r):
            with lock:
                if r.finished_s != r.finished_s:  # NaN: not yet finished
                    r.finished_s = self.clock() - start

        def work(group):
            try:
                self.runner(group, finished)
            except Exception as e:  # reported per request
                for r in group:
                    if r.error is None:
                        r.error = repr(e)
            finally:
                with lock:
                    for r in group:
                        if r.finished_s != r.finished_s:
                            r.finished_s = self.clock() - start
                        in_use[0] -= self.footprint(r.ncells)
                    running[0] -= 1
                    lock.notify_all()

        i = 0
        with ThreadPoolExecutor(self.slots) as pool:
            while i < len(reqs):
                with lock:
                    now = self.clock() - start
                    if reqs[i].arrival_s > now:
                        lock.wait(timeout=reqs[i].arrival_s - now)
                        continue
                    if running[0] >= self.slots:
                        lock.wait(timeout=0.05)
                        continue
                    # the arrived requests that wait, consecutive in arrival
                    # order, one size class, within the budget
                    cls, cap = size_class(reqs[i]), (1 if size_class(reqs[i]) else self.cohort)
                    group, need = [], 0.0
                    j = i
                    while (j < len(reqs) and len(group) < cap and reqs[j].arrival_s <= now
                           and size_class(reqs[j]) == cls
                           and in_use[0] + need + self.footprint(reqs[j].ncells) <= self.budget):
                        need += self.footprint(reqs[j].ncells)
                        group.append(reqs[j])
                        j += 1
                    if not group:
                        lock.wait(timeout=0.05)
                        continue
                    in_use[0] += need
                    running[0] += 1
                    self.peak_in_use = max(self.peak_in_use, in_use[0])
                    self.peak_running = max(self.peak_running, running[0])
                    for r in group:
                        r.admitted_s = now
                    self.cohorts.append(len(group))
                pool.submit(work, group)
                i = j
        return reqs


def make_requests(n: int, rate_per_s: float, nsteps: int = 24, large_fraction: float = 0.05, seed: int = 0):
    """Poisson arrivals at ``rate_per_s``; sizes and parameters as the batched
    instances (nx, ny ~ U{1..8}, nz ~ U{10..100}, dz ~ U(0.05, 0.5) m, log10 k
    ~ N(-12, 1), porosity ~ U(0.05, 0.35), alpha ~ logU(1e-5, 1e-3), m ~
    U(0.2, 0.6)), ``large_fraction`` of them 64 x 64 x 50 cells; top flux per
    step ~ N(0, 1e-7 m/s)."""
    r = np.random.default_rng(20261203 + seed)
    t = np.cumsum(r.exponential(1.0 / rate_per_s, n))
    out = []
    for i in range(n):
        large = r.uniform() < large_fraction
        nx, ny, nz = (64, 64, 50) if large else (int(r.integers(1, 9)), int(r.integers(1, 9)), int(r.integers(10, 101)))
        out.append(Request(rid=i, arrival_s=float(t[i]), nx=nx, ny=ny, nz=nz, dz=float(r.uniform(0.05, 0.5)),
                           k=float(10.0 ** r.normal(-12.0, 1.0)), porosity=float(r.uniform(0.05, 0.35)),
                           alpha=float(10.0 ** r.uniform(-5.0, -3.0)), m=float(r.uniform(0.2, 0.6)),
                           forcing=r.normal(0.0, 1e-7, nsteps)))
    return out


def summary(reqs, wall_s: float):
    """Latency percentiles over the requests that completed; solves/s counts
    converged solves only (a request ends at its first unconverged step)."""
    lat = np.array([r.latency_s for r in reqs if r.error is None])
    steps = sum(r.converged_steps for r in reqs)
    attempted = sum(len(r.rel_residual) for r in reqs)
    errs = [f"{r.rid}: {r.error}" for r in reqs if r.error is not None]
    setup = np.array([r.setup_s for r in reqs if np.isfinite(r.setup_s)])
    small = np.array([r.setup_s for r in reqs if np.isfinite(r.setup_s) and r.ncells < 100_000])
    large = np.array([r.setup_s for r in reqs if np.isfinite(r.setup_s) and r.ncells >= 100_000])
    return {"requests": len(reqs), "errors": len(errs), "error_messages": errs[:3],
            "step_test_steps": sum(r.step_test_steps for r in reqs),
            "setup_s_per_request": {"mean": float(setup.mean()) if setup.size else None,
                                    "p50_small": float(np.percentile(small, 50)) if small.size else None,
                                    "p50_large": float(np.percentile(large, 50)) if large.size else None},
            "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
            "solves_per_s": steps / wall_s, "converged_solves": steps, "solves_attempted": attempted,
            "solves_requested": sum(len(r.forcing) for r in reqs),
            "max_rel_residual": float(max((max(r.rel_residual) for r in reqs if r.rel_residual), default=0.0)),
            "wall_s": wall_s}
