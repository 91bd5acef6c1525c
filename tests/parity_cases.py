"""Seeded parity cases shared by the GPU parity tests and smoke().

Each case returns (tdy_configured_not_setup, U, U_prev, U_t).  States mix
saturated and unsaturated cells so every branch of the constitutive relations
(van Genuchten / Gardner saturation, Mualem cubic-smoothed / unsmoothed and
Irmay relative permeability, exponential density below/above Pref) and of the
upwinding (internal, boundary, seepage) is exercised.
"""
import numpy as np

import tdycore_gb300 as T
from tdycore_gb300 import workloads as W

PREF = 101325.0

# options inserted after every case's options_clear(); the parity tests set
# it to select the Jacobian arithmetic
EXTRA_OPTIONS = ""


def _clear():
    T.options_clear()
    if EXTRA_OPTIONS:
        T.options_insert(EXTRA_OPTIONS)


def _states(n, rng, center, spread):
    U = center + rng.normal(0.0, spread, n)
    Uprev = U + rng.normal(0.0, 0.1 * spread, n)
    Ut = rng.normal(0.0, 5.0, n)
    return U, Uprev, Ut


def case_column():
    _clear()
    t = W.box_column(1, 1, 15)
    rng = np.random.default_rng(1)
    return (t, *_states(15, rng, 102325.0, 3e3))


def case_tpf_dirichlet():
    _clear()
    t = W.box_column(5, 5, 5, gmatrix=T.MPFAO_GMATRIX_TPF, bc_type=T.DIRICHLET_BC,
                     pfunc=lambda x, y, z: 110000.0 if z > 0.99 else 100000.0)
    rng = np.random.default_rng(2)
    return (t, *_states(125, rng, 98000.0, 8e3))


def case_seepage():
    _clear()
    t = W.box_column(4, 3, 5, bc_type=T.SEEPAGE_BC, pfunc=lambda x, y, z: 99000.0 if x < 0.5 else 104000.0)
    rng = np.random.default_rng(3)
    return (t, *_states(60, rng, 101325.0, 6e3))


def case_neumann():
    _clear()
    t = W.box_column(3, 3, 3, density=T.WATER_DENSITY_CONSTANT, bc_type=T.NEUMANN_BC)
    rng = np.random.default_rng(4)
    return (t, *_states(27, rng, 95000.0, 5e3))


def case_single_cell():
    _clear()
    t = W.box_column(1, 1, 1, pfunc=lambda x, y, z: 100500.0)
    rng = np.random.default_rng(5)
    return (t, *_states(1, rng, 101000.0, 1e3))


def case_spe10_small():
    _clear()
    t, U, _ = W.spe10_like(12, 10, 8, lx=73.152, ly=30.48, lz=4.8768, seed_offset=7)
    rng = np.random.default_rng(6)
    n = U.size
    return (t, U + rng.normal(0, 2e3, n), U, rng.normal(0, 5.0, n))


def case_wedge():
    _clear()
    t, U, _ = W.wedge_extruded(npts=40, nlayers=3, seed_offset=1)
    rng = np.random.default_rng(7)
    n = U.size
    return (t, U, U + rng.normal(0, 500.0, n), rng.normal(0, 5.0, n))


def case_mixed_curves():
    """Gardner saturation and Irmay kr on some cells, Batzle-Wang EOS."""
    _clear()
    t = W.box_column(4, 4, 4, density=T.WATER_DENSITY_BATZLE_AND_WANG)
    t.set_water_viscosity_type(T.WATER_VISCOSITY_BATZLE_AND_WANG)
    cells = np.arange(0, 64, 3)
    t.set_gardner_values(np.full(cells.size, 0.5), np.full(cells.size, 0.8), np.full(cells.size, 2e-4), cells)
    cells2 = np.arange(1, 64, 4)
    t.set_irmay_values(np.full(cells2.size, 3.0), cells2)
    t.set_source_sink_values(np.linspace(-1e-3, 1e-3, 64))
    rng = np.random.default_rng(8)
    return (t, *_states(64, rng, 99000.0, 6e3))


def case_hydrostatic_box():
    _clear()
    t, U0, _ = W.hydrostatic_box(10)
    rng = np.random.default_rng(9)
    n = U0.size
    return (t, U0 + rng.normal(0, 300.0, n), U0, rng.normal(0, 2.0, n))


CASES = {
    "column": case_column,
    "tpf_dirichlet": case_tpf_dirichlet,
    "seepage": case_seepage,
    "neumann": case_neumann,
    "single_cell": case_single_cell,
    "spe10_small": case_spe10_small,
    "wedge": case_wedge,
    "mixed_curves": case_mixed_curves,
    "hydrostatic_box": case_hydrostatic_box,
}
