"""Time integration over the GPU MPFA-O residual and Jacobian.

Host-side restatement of the reference's driver path and of the PETSc
defaults it relies on, so that a run reproduces the reference's regression
output:

* ``TimeIntegrator`` follows ``TDyTimeIntegratorCreate`` /
  ``TDyTimeIntegratorRunToTime`` / ``TDyTimeIntegratorUpdateDT`` /
  ``TDyTimeIntegratorSetTargetTime`` (src/tdyti.c:8-177): options
  ``-tdy_final_time``, ``-tdy_dt_max``, ``-tdy_dt_init``,
  ``-tdy_dt_growth_factor``, ``-tdy_dt_reduction_factor``,
  ``-tdy_time_integration_method`` with the reference's defaults; a failed
  nonlinear solve cuts dt by 4 up to 25 times (the reference's MPFA_O branch
  of ``TDyTimeCut``, src/tdycore.c:2126-2140, raises "not implemented"
  instead, so there any failure ends the run).
* ``SNESNewtonLS`` restates PETSc v3.17 ``SNESSolve_NEWTONLS`` with the
  default backtracking line search (``SNESLineSearchApply_BT``, cubic order,
  alpha 1e-4, minlambda 1e-12, maxstep 1e8) and ``SNESConvergedDefault``
  (rtol 1e-8, abstol 1e-50, stol 1e-8, max_it 50, max_funcs 10000, divtol
  1e4), which ``TDyRichardsConvergenceTest`` (src/tdyrichards.c:73-93) calls.
  The Newton system is solved directly (sparse LU), as ``-pc_type lu`` does.
* ``initialize`` follows ``TDyDriverInitializeTDy`` and
  ``TDyRichardsInitialize`` (src/tdydriver.c:10-233, src/tdyrichards.c:5-28)
  for the initial condition: ``-tdy_init_file`` (PETSc binary Vec),
  ``-tdy_init_with_random_field`` (uniform in [1e4, 1e6]; PETSc's generator
  is not reproduced, so such runs are not bit-comparable), else 101325 Pa.

The residual and Jacobian come from the ``TDy`` handle (GPU; host buffers
through the C-ABI).  Any object with the same methods can stand in for it.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import MPFA_O, MPFA_O_DAE, MPFA_O_TRANSIENTVAR, options_get_real, options_get_string, options_has_name

# SNESConvergedReason values (PETSc include/petscsnes.h)
CONVERGED_FNORM_ABS = 2
CONVERGED_FNORM_RELATIVE = 3
CONVERGED_SNORM_RELATIVE = 4
CONVERGED_ITERATING = 0
DIVERGED_FUNCTION_COUNT = -2
DIVERGED_LINEAR_SOLVE = -3
DIVERGED_FNORM_NAN = -4
DIVERGED_MAX_IT = -5
DIVERGED_LINE_SEARCH = -6
DIVERGED_DTOL = -9

PETSC_VEC_CLASSID = 1211214


# ---------------------------------------------------------------------------
# PETSc binary Vec format (VecView/VecLoad with a binary viewer): big-endian
# int32 class id, int32 length, then big-endian float64 values.
def read_petsc_vec(path_or_bytes) -> np.ndarray:
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    if len(data) < 8:
        raise ValueError("PETSc binary Vec: file too short")
    classid, n = struct.unpack(">ii", data[:8])
    if classid != PETSC_VEC_CLASSID:
        raise ValueError(f"PETSc binary Vec: class id {classid}, expected {PETSC_VEC_CLASSID}")
    if n < 0 or len(data) < 8 + 8 * n:
        raise ValueError(f"PETSc binary Vec: length {n} does not fit the {len(data)}-byte file")
    return np.frombuffer(data, dtype=">f8", count=n, offset=8).astype(np.float64)


def write_petsc_vec(path, x) -> None:
    x = np.ascontiguousarray(x, dtype=np.float64)
    with open(path, "wb") as f:
        f.write(struct.pack(">ii", PETSC_VEC_CLASSID, x.size))
        f.write(x.astype(">f8").tobytes())


# ---------------------------------------------------------------------------
@dataclass
class SNESResult:
    x: np.ndarray
    reason: int
    iterations: int
    function_evaluations: int


class SNESNewtonLS:
    """Newton with backtracking line search (PETSc SNESNEWTONLS defaults)."""

    def __init__(self, rtol=1e-8, atol=1e-50, stol=1e-8, max_it=50, max_funcs=10000, divtol=1e4,
                 alpha=1e-4, minlambda=1e-12, maxstep=1e8, ls_max_it=40):
        self.rtol, self.atol, self.stol = rtol, atol, stol
        self.max_it, self.max_funcs, self.divtol = max_it, max_funcs, divtol
        self.alpha, self.minlambda, self.maxstep, self.ls_max_it = alpha, minlambda, maxstep, ls_max_it

    def _converged(self, it, xnorm, snorm, fnorm):
        # SNESConvergedDefault
        if it == 0:
            self._ttol = fnorm * self.rtol
            self._rnorm0 = fnorm
        reason = CONVERGED_ITERATING
        if not math.isfinite(fnorm):
            reason = DIVERGED_FNORM_NAN
        elif fnorm < self.atol:
            reason = CONVERGED_FNORM_ABS
        elif self._nfuncs >= self.max_funcs >= 0:
            reason = DIVERGED_FUNCTION_COUNT
        if it and not reason:
            if fnorm <= self._ttol:
                reason = CONVERGED_FNORM_RELATIVE
            elif snorm < self.stol * xnorm:
                reason = CONVERGED_SNORM_RELATIVE
            elif self.divtol > 0 and fnorm > self.divtol * self._rnorm0:
                reason = DIVERGED_DTOL
        return reason

    def _func(self, residual, x):
        self._nfuncs += 1
        return residual(x)

    def _line_search(self, residual, A, x, f, fnorm, y):
        """SNESLineSearchApply_BT (cubic).  Returns (ok, x_new, f_new,
        xnorm, gnorm, ynorm)."""
        alpha = self.alpha
        lam = 1.0
        ynorm = float(np.linalg.norm(y))
        xnorm = float(np.linalg.norm(x))
        if ynorm == 0.0:
            return False, x, f, xnorm, fnorm, ynorm
        if ynorm > self.maxstep:
            y = y * (self.maxstep / ynorm)
            ynorm = self.maxstep
        fsq = fnorm * fnorm
        initslope = float(np.dot(f, A @ y))
        if initslope > 0.0:
            initslope = -initslope
        if initslope == 0.0:
            initslope = -1.0
        while True:
            w = x - lam * y
            if self._nfuncs >= self.max_funcs:
                self._reason = DIVERGED_FUNCTION_COUNT
                return False, x, f, xnorm, fnorm, ynorm
            g_vec = self._func(residual, w)
            gnorm = float(np.linalg.norm(g_vec))
            g = gnorm * gnorm
            if math.isfinite(g):
                break
            lam *= 0.5
        if 0.5 * g <= 0.5 * fsq + lam * alpha * initslope:
            pass  # sufficient decrease with the full step
        else:
            if self.stol * xnorm > ynorm:
                return False, x, f, xnorm, fnorm, ynorm
            # quadratic fit
            lamtemp = -initslope / (g - fsq - 2.0 * lam * initslope)
            lamprev, gprev = lam, g
            if lamtemp > 0.5 * lam:
                lamtemp = 0.5 * lam
            lam = 0.1 * lam if lamtemp <= 0.1 * lam else lamtemp
            w = x - lam * y
            if self._nfuncs >= self.max_funcs:
                self._reason = DIVERGED_FUNCTION_COUNT
                return False, x, f, xnorm, fnorm, ynorm
            g_vec = self._func(residual, w)
            gnorm = float(np.linalg.norm(g_vec))
            g = gnorm * gnorm
            if not math.isfinite(g):
                return False, x, f, xnorm, fnorm, ynorm
            if not (0.5 * g < 0.5 * fsq + lam * alpha * initslope):
                # cubic fits
                count = 0
                while count < self.ls_max_it:
                    if lam <= self.minlambda:
                        return False, x, f, xnorm, fnorm, ynorm
                    t1 = 0.5 * (g - fsq) - lam * initslope
                    t2 = 0.5 * (gprev - fsq) - lamprev * initslope
                    a = (t1 / (lam * lam) - t2 / (lamprev * lamprev)) / (lam - lamprev)
                    b = (-lamprev * t1 / (lam * lam) + lam * t2 / (lamprev * lamprev)) / (lam - lamprev)
                    d = b * b - 3 * a * initslope
                    if d < 0.0:
                        d = 0.0
                    lamtemp = -initslope / (2.0 * b) if a == 0.0 else (-b + math.sqrt(d)) / (3.0 * a)
                    lamprev, gprev = lam, g
                    if lamtemp > 0.5 * lam:
                        lamtemp = 0.5 * lam
                    lam = 0.1 * lam if lamtemp <= 0.1 * lam else lamtemp
                    w = x - lam * y
                    if self._nfuncs >= self.max_funcs:
                        self._reason = DIVERGED_FUNCTION_COUNT
                        return False, x, f, xnorm, fnorm, ynorm
                    g_vec = self._func(residual, w)
                    gnorm = float(np.linalg.norm(g_vec))
                    g = gnorm * gnorm
                    if not math.isfinite(g):
                        return False, x, f, xnorm, fnorm, ynorm
                    if 0.5 * g < 0.5 * fsq + lam * alpha * initslope:
                        break
                    count += 1
                if count >= self.ls_max_it:
                    return False, x, f, xnorm, fnorm, ynorm
        return True, w, g_vec, float(np.linalg.norm(w)), gnorm, ynorm

    def solve(self, residual, jacobian, x, rowptr, colidx) -> SNESResult:
        """``residual(x)`` -> F; ``jacobian(x)`` -> CSR values over (rowptr,
        colidx)."""
        n = x.size
        x = np.array(x, dtype=np.float64)
        self._nfuncs = 0
        self._reason = CONVERGED_ITERATING
        f = self._func(residual, x)
        fnorm = float(np.linalg.norm(f))
        if not math.isfinite(fnorm):
            return SNESResult(x, DIVERGED_FNORM_NAN, 0, self._nfuncs)
        reason = self._converged(0, 0.0, 0.0, fnorm)
        if reason:
            return SNESResult(x, reason, 0, self._nfuncs)
        for i in range(self.max_it):
            A = sp.csr_matrix((jacobian(x), colidx, rowptr), shape=(n, n))
            try:
                y = spla.spsolve(A.tocsc(), f)
            except RuntimeError:
                return SNESResult(x, DIVERGED_LINEAR_SOLVE, i, self._nfuncs)
            if not np.all(np.isfinite(y)):
                return SNESResult(x, DIVERGED_LINEAR_SOLVE, i, self._nfuncs)
            ok, x_new, f_new, xnorm, fnorm_new, ynorm = self._line_search(residual, A, x, f, fnorm, y)
            if self._reason == DIVERGED_FUNCTION_COUNT:
                return SNESResult(x, DIVERGED_FUNCTION_COUNT, i, self._nfuncs)
            if not ok:
                if self.stol * xnorm > ynorm:
                    return SNESResult(x, CONVERGED_SNORM_RELATIVE, i, self._nfuncs)
                return SNESResult(x, DIVERGED_LINE_SEARCH, i, self._nfuncs)
            x, f, fnorm = x_new, f_new, fnorm_new
            reason = self._converged(i + 1, xnorm, ynorm, fnorm)
            if reason:
                return SNESResult(x, reason, i + 1, self._nfuncs)
        return SNESResult(x, DIVERGED_MAX_IT, self.max_it, self._nfuncs)


# ---------------------------------------------------------------------------
# Jacobian of the DAE form over interleaved unknowns [P_0, M_0, P_1, M_1, ...]:
# row 2i holds the flux row of cell i (columns 2j) plus column 2i+1; row 2i+1
# holds columns 2i and 2i+1.
def dae_pattern(t):
    cache = getattr(t, "_dae_pattern", None)
    if cache is not None:
        return cache
    n, rp, ci = t.ncells, t.rowptr, t.colidx
    counts = np.empty(2 * n, dtype=np.int64)
    counts[0::2] = np.diff(rp) + 1
    counts[1::2] = 2
    rp2 = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    ci2 = np.empty(rp2[-1], dtype=np.int32)
    for i in range(n):
        a = rp2[2 * i]
        cols = np.concatenate([2 * ci[rp[i]:rp[i + 1]], [2 * i + 1]])
        ci2[a:a + cols.size] = np.sort(cols)
        ci2[rp2[2 * i + 1]:rp2[2 * i + 1] + 2] = (2 * i, 2 * i + 1)
    t._dae_pattern = (rp2, ci2, t.cell_volumes())
    return t._dae_pattern


def dae_values(t, Jflux, dRp_dM, dRm_dP, dRm_dM):
    n, rp, ci = t.ncells, t.rowptr, t.colidx
    rp2, ci2, _ = dae_pattern(t)
    vals = np.empty(rp2[-1])
    for i in range(n):
        a, b = rp[i], rp[i + 1]
        cols = ci[a:b]
        k = int(np.searchsorted(2 * cols, 2 * i + 1))  # position of column 2i+1 among the sorted row
        base = rp2[2 * i]
        vals[base:base + k] = Jflux[a:a + k]
        vals[base + k] = dRp_dM[i]
        vals[base + k + 1:base + (b - a) + 1] = Jflux[a + k:b]
        vals[rp2[2 * i + 1]] = dRm_dP[i]
        vals[rp2[2 * i + 1] + 1] = dRm_dM[i]
    return vals


def initial_condition(ncells: int, seed: int = 0) -> np.ndarray:
    """TDyRichardsInitialize (src/tdyrichards.c:5-28) from the options."""
    init_file = options_get_string("-tdy_init_file")
    random_field = options_has_name("-tdy_init_with_random_field")
    if init_file and random_field:
        raise ValueError("Only one of -tdy_init_from_file and -tdy_init_with_random_field can be specified")
    if random_field:
        return np.random.default_rng(seed).uniform(1.0e4, 1.0e6, ncells)
    if init_file:
        u = read_petsc_vec(init_file)
        if u.size != ncells:
            raise ValueError(f"{init_file}: {u.size} values for {ncells} cells")
        return u
    return np.full(ncells, 101325.0)


class TimeIntegrator:
    """TDyTimeIntegrator (src/tdyti.c) driving a TDy handle."""

    SNES, TS = "SNES", "TS"

    def __init__(self, tdy, snes: SNESNewtonLS | None = None):
        self.tdy = tdy
        self.snes = snes or SNESNewtonLS()
        self.method = self.SNES
        self.dt_init = 1.0
        self.dt_max = 1.0e20
        self.dt_growth_factor = 1.25
        self.dt_reduction_factor = 0.5
        self.time = 0.0
        self.dt_save = 0.0
        self.final_time = 0.0001 * 365.0 * 24.0 * 3600.0
        self.istep = 0
        self.max_time_step_cuts = 25
        self.final_time = options_get_real("-tdy_final_time", self.final_time)
        self.dt_max = options_get_real("-tdy_dt_max", self.dt_max)
        self.dt_init = options_get_real("-tdy_dt_init", self.dt_init)
        self.dt_growth_factor = options_get_real("-tdy_dt_growth_factor", self.dt_growth_factor)
        self.dt_reduction_factor = options_get_real("-tdy_dt_reduction_factor", self.dt_reduction_factor)
        m = options_get_string("-tdy_time_integration_method")
        if m:
            if m not in (self.SNES, self.TS):
                raise ValueError("Unrecognized Time Integration Method")
            self.method = m
        self.dt = self.dt_init
        self.soln = None
        self.history = []  # (istep, time, dt, newton its, reason)

    def set_solution(self, U):
        """TDySetInitialCondition: the solution and the previous solution."""
        self.soln = np.array(U, dtype=np.float64)
        self.tdy.set_previous_solution(self.soln)

    def set_time_step(self, dt):
        """TDyTimeIntegratorSetTimeStep (src/tdyti.c:92-98)."""
        self.dt_init = dt
        self.dt = dt

    def _update_dt(self, sync_time):
        if self.dt_save > 0.0:
            self.time = sync_time
            self.dt = self.dt_save
            self.dt_save = 0.0
        self.dt *= self.dt_growth_factor
        if self.dt > self.dt_max:
            self.dt = self.dt_max

    def _set_target_time(self, sync_time):
        dt_for_sync = sync_time - self.time
        if self.dt > dt_for_sync:
            self.dt_save = self.dt
            self.dt = dt_for_sync

    def _snes_step(self):
        t = self.tdy
        return self.snes.solve(t.snes_function, t.snes_jacobian, self.soln.copy(), t.rowptr, t.colidx)

    def run_to_time(self, sync_time):
        """TDyTimeIntegratorRunToTime (src/tdyti.c:100-177)."""
        t = self.tdy
        if self.method == self.SNES:
            icut = 0
            while self.time < sync_time:
                self._set_target_time(sync_time)
                t.set_dtime(self.dt)
                while True:
                    t.presolve_current()
                    res = self._snes_step()
                    if res.reason < 0:
                        icut += 1
                        self.dt *= 0.25
                        t.set_dtime(self.dt)
                        self.history.append((self.istep, self.time, self.dt, res.iterations, res.reason))
                        if icut == self.max_time_step_cuts:
                            raise RuntimeError("TDyTimeIntegratorRunToTime failed to converge after maximum "
                                               "time step cuts")
                        continue
                    self.time += self.dt
                    self.istep += 1
                    self.soln = res.x
                    t.post_solve(self.soln)
                    self.history.append((self.istep, self.time, self.dt, res.iterations, res.reason))
                    break
                self._update_dt(sync_time)
        else:
            # PETSc TSBEULER, fixed step dt_init, TS_EXACTFINALTIME_MATCHSTEP,
            # with the IFunction of the handle's discretization
            tmax = sync_time - self.time
            dt = self.dt_init
            tt = 0.0
            while tmax - tt > 1e-12 * max(1.0, abs(tmax)):
                h = min(dt, tmax - tt)
                res = self._ts_beuler_step(self.time + tt + h, h)
                if res.reason < 0:
                    raise RuntimeError(f"TS step failed: SNES reason {res.reason}")
                self.soln = res.x
                tt += h
                self.istep += 1
                self.history.append((self.istep, self.time + tt, h, res.iterations, res.reason))
            self.time += tt
            dae = getattr(t, "discretization", MPFA_O) == MPFA_O_DAE
            t.post_solve(self.soln[0::2] if dae else self.soln)
        return self.soln

    def _ts_beuler_step(self, time, h):
        """One backward-Euler step of the handle's TS form: F(t, U, (U - U_n)/h)
        = 0 (TDyMPFAOIFunction), its transient-variable form with
        M_t = (C(U) - C(U_n))/h (TDyMPFAOIFunction_TransientVariable), or the
        DAE form over interleaved [P, M] (TDyMPFAOIFunction_DAE)."""
        t = self.tdy
        U0 = self.soln.copy()
        disc = getattr(t, "discretization", MPFA_O)
        if disc == MPFA_O_TRANSIENTVAR:
            C0 = t.transient_variable(U0)
            return self.snes.solve(lambda x: t.tv_ifunction(time, x, (t.transient_variable(x) - C0) / h),
                                   lambda x: t.tv_ijacobian(time, x, 1.0 / h), U0.copy(), t.rowptr, t.colidx)
        if disc == MPFA_O_DAE:
            rp, ci, vol = dae_pattern(t)
            n = t.ncells

            def jac(x):
                # [dR_P/dP  dR_P/dM; dR_M/dP  dR_M/dM] = [fluxes  V/h; -dC/dP  1]
                P = x[0::2]
                Jf = t.tv_ijacobian(time, P, 0.0)
                _, dC = t.transient_variable(P, with_derivative=True)
                return dae_values(t, Jf, vol / h, -dC, np.ones(n))

            return self.snes.solve(lambda x: t.dae_ifunction(time, x, (x - U0) / h), jac, U0.copy(), rp, ci)
        return self.snes.solve(lambda x: t.ifunction(time, x, (x - U0) / h),
                               lambda x: t.ijacobian(time, x, (x - U0) / h, 1.0 / h), U0.copy(), t.rowptr,
                               t.colidx)

    def output_regression(self):
        """TDyTimeIntegratorOutputRegression: regression file of the previous
        solution, which equals the current one after TDyPostSolve."""
        self.tdy.output_regression(self.soln)


def initialize(tdy, seed: int = 0) -> TimeIntegrator:
    """TDyDriverInitializeTDy for the MPFA-O Richards path: TDySetup, the
    time integrator from the options, the initial condition."""
    if not tdy.ncells:
        tdy.setup()
    ti = TimeIntegrator(tdy)
    ti.set_solution(initial_condition(tdy.ncells, seed))
    return ti
