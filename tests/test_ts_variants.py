"""TS variants on the same flux kernels: the transient-variable form
(tdympfao_ts_transientvar.c) and the DAE form over interleaved [P, M]
(tdympfao_ts_dae.c).

GPU parity against the oracle for every entry point, and a property that ties
the variants to the pinned SNES form: with backward Euler and no source, the
transient-variable residual with M_t = (C(U) - C(U_n))/dt and the DAE
residual (M = C(P), M_t = (M - M_n)/dt) have the same discrete solution as the
SNES form, whose runs reproduce the reference's regression golds.
"""
import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300 import driver as D
from tdycore_gb300.workloads import box_column
from oracle import Oracle
from tests.parity_cases import CASES

DT = 600.0


class OracleForms:
    """The handle methods the driver's TS step calls, from the oracle."""

    def __init__(self, t, disc):
        self.t, self.o = t, Oracle(t.setup_view())
        self.ncells, self.nnz = t.ncells, t.nnz
        self.rowptr, self.colidx = t.rowptr, t.colidx
        self.discretization = disc

    def cell_volumes(self):
        return self.t.cell_volumes()

    def transient_variable(self, U, with_derivative=False):
        return self.o.transient_variable(U, with_derivative)

    def tv_ifunction(self, time, U, M_t):
        return self.o.tv_ifunction(U, M_t)

    def tv_ijacobian(self, time, U, shift):
        return self.o.tv_ijacobian(U, shift)

    def dae_ifunction(self, time, U, U_t):
        return self.o.dae_ifunction(U, U_t)

    def post_solve(self, U):
        pass


def column(disc):
    """3x3x4 column, exponential density, Dirichlet 1e5 Pa on the top face and
    no flow elsewhere (explicit boundary values: without them the reference's
    Jacobian ignores that a Dirichlet face then takes its cell's pressure, and
    Newton converges only linearly)."""
    T.options_clear()
    t = box_column(3, 3, 4, pfunc=lambda x, y, z: 1.0e5)
    t.set_boundary_pressure_type_function(lambda x, y, z: T.DIRICHLET_BC if z > 1.0 - 1e-9 else T.NEUMANN_BC)
    t.set_discretization(disc)
    return t


def snes_reference(o, U0, nsteps):
    snes = D.SNESNewtonLS(rtol=1e-10, stol=1e-12)
    U = U0.copy()
    for _ in range(nsteps):
        o.snes_presolve(U, DT)
        r = snes.solve(o.snes_function, o.snes_jacobian, U.copy(), *o.pattern())
        assert r.reason > 0
        U = r.x
    return U


def run_variant(handle, U0, nsteps):
    ti = D.TimeIntegrator(handle, D.SNESNewtonLS(rtol=1e-10, stol=1e-12))
    ti.method = ti.TS
    ti.dt_init = DT
    ti.soln = U0.copy()
    ti.run_to_time(DT * nsteps)
    return ti.soln


def initial_state(n):
    return 101325.0 + np.random.default_rng(3).normal(0.0, 4e3, n)


@pytest.mark.parametrize("disc", [T.MPFA_O_TRANSIENTVAR, T.MPFA_O_DAE])
def test_variants_match_snes_form_oracle(disc):
    t = column(disc)
    t.setup(host_only=True)
    h = OracleForms(t, disc)
    P0 = initial_state(t.ncells)
    Us = snes_reference(h.o, P0, 3)
    if disc == T.MPFA_O_DAE:
        U0 = np.stack([P0, h.o.transient_variable(P0)], axis=1).ravel()
        Uv = run_variant(h, U0, 3)[0::2]
    else:
        Uv = run_variant(h, P0, 3)
    assert np.max(np.abs(Uv - Us) / np.abs(Us)) < 1e-9


def test_discretization_variants_accepted():
    T.options_clear()
    for d in (T.MPFA_O, T.MPFA_O_DAE, T.MPFA_O_TRANSIENTVAR):
        T.create_richards_mpfao().set_discretization(d)
    with pytest.raises(T.TDyError):
        T.create_richards_mpfao().set_discretization(T.BDM)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["spe10_small", "mixed_curves", "seepage", "wedge"])
def test_variant_parity_gpu(name):
    t, U, Uprev, Ut = CASES[name]()
    t.setup()
    o = Oracle(t.setup_view())
    C, dC = t.transient_variable(U, with_derivative=True)
    Cr, dCr = o.transient_variable(U, with_derivative=True)
    assert np.allclose(C, Cr, rtol=1e-14, atol=0) and np.allclose(dC, dCr, rtol=1e-13, atol=1e-300)
    Mt = Ut * dCr  # any rate
    R = t.tv_ifunction(0.0, U, Mt)
    Rr, Rm = o.tv_ifunction(U, Mt, with_mag=True)
    assert np.all(np.abs(R - Rr) <= 1e-12 * Rm)
    J = t.tv_ijacobian(0.0, U, 1.0 / DT)
    Jr, Jm = o.tv_ijacobian(U, 1.0 / DT, with_mag=True)
    assert np.all(np.abs(J - Jr) <= 1e-10 * Jm)
    U2 = np.stack([U, Cr * 1.001], axis=1).ravel()
    Ut2 = np.stack([Ut, Mt], axis=1).ravel()
    R2 = t.dae_ifunction(0.0, U2, Ut2)
    R2r, R2m = o.dae_ifunction(U2, Ut2, with_mag=True)
    assert np.all(np.abs(R2 - R2r) <= 1e-12 * R2m)


@pytest.mark.gpu
@pytest.mark.parametrize("disc", [T.MPFA_O_TRANSIENTVAR, T.MPFA_O_DAE])
def test_variants_match_snes_form_gpu(disc):
    t = column(disc)
    t.setup()
    o = Oracle(t.setup_view())
    P0 = initial_state(t.ncells)
    Us = snes_reference(o, P0, 3)
    if disc == T.MPFA_O_DAE:
        U0 = np.stack([P0, t.transient_variable(P0)], axis=1).ravel()
        Uv = run_variant(t, U0, 3)[0::2]
    else:
        Uv = run_variant(t, P0, 3)
    assert np.max(np.abs(Uv - Us) / np.abs(Us)) < 1e-9
