"""Pin the oracle and the host setup to the reference's regression golds.

The reference's regression harness compares max/min/mean and sampled-cell
pressures after full Newton + LU runs with a 1e-12 relative tolerance
(demo/transient/*.cfg "pressure = 1.0e-12 relative").  The same runs here use
the host MPFA-O setup (mesh, transmissibility, gravity discretization) and
the C oracle's residual and Jacobian inside a restated PETSc Newton driver.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300.workloads import box_column
from oracle import Oracle
from tests.newton_ref import snes_steps, ts_beuler_steps

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


def _oracle(t):
    t.setup(host_only=True)
    return Oracle(t.setup_view())


def test_snes_default_column():
    # -max_steps 10 on the 1x1x15 column, exponential density, IC 102325
    T.options_clear()
    o = _oracle(box_column(1, 1, 15))
    U = snes_steps(o, np.full(15, 102325.0), 1800.0, 10)
    check_gold("transient-snes-mpfaof90", U)


@pytest.mark.parametrize("name,bct", [("transient-snes-mpfaof90-dirichlet", T.DIRICHLET_BC),
                                      ("transient-snes-mpfaof90-seepage", T.SEEPAGE_BC)])
def test_snes_5x5x5_tpf(name, bct):
    T.options_clear()
    o = _oracle(box_column(5, 5, 5, gmatrix=T.MPFAO_GMATRIX_TPF, bc_type=bct, pfunc=top_center_pressure))
    U = snes_steps(o, np.full(125, 90325.0), 1800.0, 48)
    check_gold(name, U)


@pytest.mark.parametrize("name,gm,bct", [("transient-mpfaof90", 0, None), ("transient-mpfaof90-tpf", 1, None),
                                         ("transient-mpfaof90-neumann", 0, T.NEUMANN_BC),
                                         ("transient-mpfaof90-tpf-neumann", 1, T.NEUMANN_BC)])
def test_ts_beuler_3x3x3(name, gm, bct):
    # demo/transient/transient_mpfaof90.F90: constant density, P_bc = 1e5, IC 90325, 10 x 100 s
    T.options_clear()
    t = box_column(3, 3, 3, density=T.WATER_DENSITY_CONSTANT, gmatrix=gm, bc_type=bct,
                   pfunc=lambda x, y, z: 100000.0)
    o = _oracle(t)
    U = ts_beuler_steps(o, np.full(27, 90325.0), 100.0, 10)
    check_gold(name, U)
