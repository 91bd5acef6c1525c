"""Pin the oracle, the host setup and the GPU path to the reference's
regression golds.

The reference's regression harness compares max/min/mean and sampled-cell
pressures after full Newton + LU runs with a 1e-12 relative tolerance
(demo/transient/*.cfg "pressure = 1.0e-12 relative").  The same runs here use
the host MPFA-O setup (mesh, transmissibility, gravity discretization) and
the package's restatement of PETSc's Newton (tdycore_gb300.driver), with the
residual and Jacobian from the C oracle (CPU) or from the GPU path.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300 import driver as D
from tdycore_gb300.workloads import box_column
from oracle import Oracle

GOLD = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())["cases"]
RTOL = 1.0e-12


def check_gold(name, U):
    g = GOLD[name]
    got = {"max": U.max(), "min": U.min(), "mean": U.mean()}
    for k in ("max", "min", "mean"):
        assert abs(got[k] - g[k]) <= RTOL * abs(g[k]), (name, k, got[k], g[k])
    for idx, val in g["sampled"].items():
        assert abs(U[int(idx)] - val) <= RTOL * abs(val), (name, idx, U[int(idx)], val)


def top_center_pressure(x, y, z):
    # PressureFunction of demo/transient/transient_snes_mpfaof90.F90:110-130
    return 110000.0 if (0.0 < x < 1.0 and 0.0 < y < 1.0 and z > 0.99) else 100000.0


class Residuals:
    """SNES and TS residual/Jacobian of one mesh from the oracle or the GPU."""

    def __init__(self, t, backend):
        self.backend = backend
        if backend == "gpu":
            t.setup()
            self.t = t
        else:
            t.setup(host_only=True)
            self.o = Oracle(t.setup_view())
        self.rowptr, self.colidx = t.rowptr, t.colidx

    def presolve(self, U, dt):
        if self.backend == "gpu":
            self.t.set_dtime(dt)
            self.t.presolve(U)
        else:
            self.o.snes_presolve(U, dt)

    def F(self, U):
        return self.t.snes_function(U) if self.backend == "gpu" else self.o.snes_function(U)

    def J(self, U):
        return self.t.snes_jacobian(U) if self.backend == "gpu" else self.o.snes_jacobian(U)

    def IF(self, U, Ut):
        return self.t.ifunction(0.0, U, Ut) if self.backend == "gpu" else self.o.ts_ifunction(U, Ut)

    def IJ(self, U, Ut, shift):
        return self.t.ijacobian(0.0, U, Ut, shift) if self.backend == "gpu" else self.o.ts_ijacobian(U, Ut, shift)


def snes_steps(r, U, dt, nsteps):
    """Backward Euler with the SNES form: TDyPreSolveSNESSolver + SNESSolve
    per step, as demo/transient/transient_snes_mpfaof90.F90 does."""
    snes = D.SNESNewtonLS()
    for _ in range(nsteps):
        r.presolve(U, dt)
        res = snes.solve(r.F, r.J, U.copy(), r.rowptr, r.colidx)
        assert res.reason > 0, res
        U = res.x
    return U


def ts_beuler_steps(r, U, dt, nsteps):
    """TSBEULER with IFunction/IJacobian: F(U, (U - U_n)/dt) = 0, shift 1/dt."""
    snes = D.SNESNewtonLS()
    for _ in range(nsteps):
        Un = U.copy()
        res = snes.solve(lambda x: r.IF(x, (x - Un) / dt), lambda x: r.IJ(x, (x - Un) / dt, 1.0 / dt),
                         U.copy(), r.rowptr, r.colidx)
        assert res.reason > 0, res
        U = res.x
    return U


BACKENDS = ["oracle", pytest.param("gpu", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("backend", BACKENDS)
def test_snes_default_column(backend):
    # -max_steps 10 on the 1x1x15 column, exponential density, IC 102325
    T.options_clear()
    r = Residuals(box_column(1, 1, 15), backend)
    U = snes_steps(r, np.full(15, 102325.0), 1800.0, 10)
    check_gold("transient-snes-mpfaof90", U)


@pytest.mark.parametrize("backend", BACKENDS)
@pytest.mark.parametrize("name,bct", [("transient-snes-mpfaof90-dirichlet", T.DIRICHLET_BC),
                                      ("transient-snes-mpfaof90-seepage", T.SEEPAGE_BC)])
def test_snes_5x5x5_tpf(name, bct, backend):
    T.options_clear()
    r = Residuals(box_column(5, 5, 5, gmatrix=T.MPFAO_GMATRIX_TPF, bc_type=bct, pfunc=top_center_pressure), backend)
    U = snes_steps(r, np.full(125, 90325.0), 1800.0, 48)
    check_gold(name, U)


@pytest.mark.parametrize("backend", BACKENDS)
@pytest.mark.parametrize("name,gm,bct", [("transient-mpfaof90", 0, None), ("transient-mpfaof90-tpf", 1, None),
                                         ("transient-mpfaof90-neumann", 0, T.NEUMANN_BC),
                                         ("transient-mpfaof90-tpf-neumann", 1, T.NEUMANN_BC)])
def test_ts_beuler_3x3x3(name, gm, bct, backend):
    # demo/transient/transient_mpfaof90.F90: constant density, P_bc = 1e5, IC 90325, 10 x 100 s
    T.options_clear()
    t = box_column(3, 3, 3, density=T.WATER_DENSITY_CONSTANT, gmatrix=gm, bc_type=bct,
                   pfunc=lambda x, y, z: 100000.0)
    r = Residuals(t, backend)
    U = ts_beuler_steps(r, np.full(27, 90325.0), 100.0, 10)
    check_gold(name, U)
