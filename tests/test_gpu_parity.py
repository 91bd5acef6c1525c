"""GPU residual/Jacobian parity with the oracle (C restatement of the reference).

Tolerances (FP64):
  residual:  |R_gpu - R_ref| <= 1e-12 * sum_k |terms_k into cell i|  (per cell)
  Jacobian:  |J_gpu - J_ref| <= 1e-10 * sum_k |contributions_k|      (per entry)
The right-hand sides are the floating-point error scale of each summed
quantity (the oracle accumulates the absolute values of every term it adds),
so cancellation near equilibrium does not make the bar meaningless.  The CSR
pattern must match the oracle's independently computed pattern bit for bit.
"""
import numpy as np
import pytest

from oracle import Oracle
from tests import parity_cases
from tests.parity_cases import CASES

pytestmark = pytest.mark.gpu

R_TOL = 1e-12
J_TOL = 1e-10
DT = 1800.0


# Jacobian products at interior hexahedral vertices: double-float (default)
# or FP64; both must meet the same bars
ARITH = ["DOUBLE_FLOAT", "FP64"]


def _setup(name, arith="DOUBLE_FLOAT"):
    parity_cases.EXTRA_OPTIONS = f"-tdy_jacobian_arithmetic {arith}"
    try:
        t, U, Uprev, Ut = CASES[name]()
    finally:
        parity_cases.EXTRA_OPTIONS = ""
    t.setup()
    o = Oracle(t.setup_view())
    return t, o, U, Uprev, Ut


def assert_close(got, ref, mag, tol, what):
    err = np.abs(got - ref)
    bound = tol * np.maximum(mag, np.finfo(float).tiny)
    bad = np.nonzero(err > bound)[0]
    assert bad.size == 0, (f"{what}: {bad.size} entries out of tolerance; worst index {bad[np.argmax(err[bad] / bound[bad])]}"
                           f" err {err[bad].max():.3e} mag {mag[bad].max():.3e}")


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("name", list(CASES))
def test_snes_parity(name, arith):
    t, o, U, Uprev, _ = _setup(name, arith)
    rp, ci = o.pattern()
    assert np.array_equal(rp, t.rowptr) and np.array_equal(ci, t.colidx), "CSR pattern differs"
    t.set_dtime(DT)
    t.presolve(Uprev)
    o.snes_presolve(Uprev, DT)
    R, J = t.snes_function_jacobian(U)
    Rr, Rm = o.snes_function(U, with_mag=True)
    Jr, Jm = o.snes_jacobian(U, with_mag=True)
    assert_close(R, Rr, Rm, R_TOL, f"{name} SNES residual")
    assert_close(J, Jr, Jm, J_TOL, f"{name} SNES Jacobian")
    # norm-wise at these perturbed, non-equilibrium states
    assert np.linalg.norm(R - Rr) <= R_TOL * np.linalg.norm(Rr), f"{name}: ||dR||/||R|| above {R_TOL}"
    # separate entry points agree with the fused one bit for bit
    assert np.array_equal(t.snes_function(U), R)
    assert np.array_equal(t.snes_jacobian(U), J)


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("name", list(CASES))
def test_ts_parity(name, arith):
    t, o, U, _, Ut = _setup(name, arith)
    shift = 1.0 / 100.0
    R, J = t.ifunction_ijacobian(0.0, U, Ut, shift)
    Rr, Rm = o.ts_ifunction(U, Ut, with_mag=True)
    Jr, Jm = o.ts_ijacobian(U, Ut, shift, with_mag=True)
    assert_close(R, Rr, Rm, R_TOL, f"{name} TS residual")
    assert_close(J, Jr, Jm, J_TOL, f"{name} TS Jacobian")


def test_deterministic_and_device_entry_point():
    import torch

    t, o, U, Uprev, _ = _setup("spe10_small")
    t.set_dtime(DT)
    t.presolve(Uprev)
    R1, J1 = t.snes_function_jacobian(U)
    R2, J2 = t.snes_function_jacobian(U)
    assert np.array_equal(R1, R2) and np.array_equal(J1, J2)
    dU = torch.tensor(U, dtype=torch.float64, device="cuda")
    dR = torch.empty(t.ncells, dtype=torch.float64, device="cuda")
    dJ = torch.empty(t.nnz, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    t.snes_function_jacobian_device(dU, dR, dJ, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dR.cpu().numpy(), R1)
    assert np.array_equal(dJ.cpu().numpy(), J1)


def test_pinned_host_buffers_slab_graph():
    """Pinned host buffers take the slab pipeline as one graph: the same bits
    as pageable buffers and the device entry point, and a changed dt (which
    the graph bakes in) gives a fresh graph with the new step's values."""
    import torch

    t, o, U, Uprev, _ = _setup("spe10_small")
    t.set_dtime(DT)
    t.presolve(Uprev)
    R1, J1 = t.snes_function_jacobian(U)
    Up = torch.tensor(U, dtype=torch.float64).pin_memory()
    Rp = torch.full((t.ncells,), np.nan, dtype=torch.float64).pin_memory()
    Jp = torch.full((t.nnz,), np.nan, dtype=torch.float64).pin_memory()
    for _ in range(2):
        t.snes_function_jacobian(Up.numpy(), Rp.numpy(), Jp.numpy())
        assert np.array_equal(Rp.numpy(), R1) and np.array_equal(Jp.numpy(), J1)
    t.set_dtime(DT / 4)
    t.presolve(Uprev)
    R2, J2 = t.snes_function_jacobian(U)
    t.snes_function_jacobian(Up.numpy(), Rp.numpy(), Jp.numpy())
    assert np.array_equal(Rp.numpy(), R2) and np.array_equal(Jp.numpy(), J2)
    assert not np.array_equal(R2, R1)
    o.snes_presolve(Uprev, DT / 4)
    Rr, Rm = o.snes_function(U, with_mag=True)
    assert_close(Rp.numpy(), Rr, Rm, R_TOL, "pinned slab graph residual")


def test_jacobian_is_derivative_of_residual():
    """Central differences of the GPU residual against the GPU Jacobian."""
    t, o, U, Uprev, _ = _setup("spe10_small")
    t.set_dtime(DT)
    t.presolve(Uprev)
    R, J = t.snes_function_jacobian(U)
    n = t.ncells
    rng = np.random.default_rng(11)
    d = rng.standard_normal(n)
    eps = 1e-3
    fd = (t.snes_function(U + eps * d) - t.snes_function(U - eps * d)) / (2 * eps)
    rows = np.repeat(np.arange(n), np.diff(t.rowptr))
    Jd = np.bincount(rows, weights=J * d[t.colidx], minlength=n)
    scale = np.abs(Jd).max()
    assert np.abs(fd - Jd).max() <= 1e-5 * scale


@pytest.mark.parametrize("name", ["spe10_small", "hydrostatic_box", "mixed_curves"])
def test_double_float_jacobian_tracks_fp64(name):
    """The double-float Jacobian products stay within 1e-12 of the error scale
    of the FP64 ones (two orders inside the parity bar); residuals are FP64 in
    both and identical."""
    runs = {}
    for arith in ARITH:
        t, o, U, Uprev, _ = _setup(name, arith)
        t.set_dtime(DT)
        t.presolve(Uprev)
        o.snes_presolve(Uprev, DT)
        runs[arith] = t.snes_function_jacobian(U)
    _, Jm = o.snes_jacobian(U, with_mag=True)
    (Rf, Jf), (Rd, Jd) = runs["DOUBLE_FLOAT"], runs["FP64"]
    assert np.array_equal(Rf, Rd)
    assert_close(Jf, Jd, Jm, 1e-12, f"{name} double-float vs FP64 Jacobian")


@pytest.mark.parametrize("name", ["spe10_small", "hydrostatic_box", "tpf_dirichlet", "mixed_curves", "seepage",
                                  "neumann", "wedge", "column", "single_cell"])
def test_device_built_transmissibility(name):
    """-tdy_mpfao_setup_on_device: Trans is built by the device kernels (the
    interior hexahedral vertices one thread each, eliminating the
    interaction-region unknowns in another order than the host; the boundary,
    prismatic and other vertices one warp each, with the host's system).
    Wedge (prism), one-column and single-cell meshes are all boundary
    vertices.  R must meet the usual bar against the oracle
    on the host-built setup.  For J the bar is taken relative to the larger of
    the entry's error scale and one FP64 unit (1e-16) of the largest scale in
    its row: entries that are structural zeros of Trans (orthogonal meshes)
    hold only rounding noise of the elimination, which two Trans computations
    produce differently."""
    parity_cases.EXTRA_OPTIONS = "-tdy_mpfao_setup_on_device"
    try:
        t, U, Uprev, Ut = CASES[name]()
    finally:
        parity_cases.EXTRA_OPTIONS = ""
    t.setup()
    th, _, _, _ = CASES[name]()
    th.setup(host_only=True)
    o = Oracle(th.setup_view())
    assert np.array_equal(t.rowptr, th.rowptr) and np.array_equal(t.colidx, th.colidx)
    t.set_dtime(DT)
    t.presolve(Uprev)
    o.snes_presolve(Uprev, DT)
    R, J = t.snes_function_jacobian(U)
    Rr, Rm = o.snes_function(U, with_mag=True)
    Jr, Jm = o.snes_jacobian(U, with_mag=True)
    assert_close(R, Rr, Rm, R_TOL, f"{name} SNES residual, device-built Trans")
    rowmax = np.maximum.reduceat(Jm, t.rowptr[:-1])
    row_of = np.repeat(np.arange(t.ncells), np.diff(t.rowptr))
    assert_close(J, Jr, np.maximum(Jm, 1e-16 * rowmax[row_of]), J_TOL, f"{name} SNES Jacobian, device-built Trans")


@pytest.mark.parametrize("name", ["spe10_small", "tpf_dirichlet", "mixed_curves", "wedge", "seepage", "column"])
def test_device_built_trans_in_setup_view(name):
    """The setup view of a handle with device-built Trans holds the device
    values; they equal the host-built ones to rounding of the row scale."""
    parity_cases.EXTRA_OPTIONS = "-tdy_mpfao_setup_on_device"
    try:
        t, _, _, _ = CASES[name]()
    finally:
        parity_cases.EXTRA_OPTIONS = ""
    t.setup()
    th, _, _, _ = CASES[name]()
    th.setup(host_only=True)
    vd, vh = t.setup_view(), th.setup_view()
    Td, Th = vd["trans"], vh["trans"]
    assert Td.shape == Th.shape
    for v in range(vh["nverts"]):
        a, b = vh["v_trans_off"][v], vh["v_trans_off"][v + 1]
        if a == b:
            continue
        scale = np.abs(Th[a:b]).max()
        assert np.all(np.abs(Td[a:b] - Th[a:b]) <= 1e-13 * scale), v


def hub_prisms(nring=42, nlayers=3):
    """Prisms over the Delaunay triangulation of three close hub points inside
    a ring of ``nring`` points: each hub has valence ~17 (within the vertex
    kernel's limits of 64 rows and 64 cells per vertex), and a wedge touching
    the hubs shares a vertex with ~46 triangles' wedges in each of three
    layers, so its Jacobian row has more than 96 entries."""
    import tdycore_gb300 as T_
    from scipy.spatial import Delaunay
    from tdycore_gb300 import workloads as W

    ang = np.linspace(0.0, 2.0 * np.pi, nring, endpoint=False)
    hub = np.linspace(0.0, 2.0 * np.pi, 3, endpoint=False) + 0.3
    xy = np.vstack([np.c_[2.0 * np.cos(hub), 2.0 * np.sin(hub)], np.c_[20.0 * np.cos(ang), 20.0 * np.sin(ang)]])
    tris = Delaunay(xy).simplices.astype(np.int32)
    P = xy[tris]
    cw = (P[:, 1, 0] - P[:, 0, 0]) * (P[:, 2, 1] - P[:, 0, 1]) - (P[:, 1, 1] - P[:, 0, 1]) * (P[:, 2, 0] - P[:, 0, 0]) < 0
    tris[cw] = tris[cw][:, [0, 2, 1]]
    z = np.repeat(np.array([0.0, 0.7, 2.0, 3.1])[:nlayers + 1, None], xy.shape[0], axis=1)
    nc = nlayers * tris.shape[0]
    rng = np.random.default_rng(41)
    T_.options_clear()
    t = T_.create_richards_mpfao()
    t.set_extruded_mesh(xy, tris, z)
    t.set_from_options()
    t.set_permeability_values(W.random_spd(nc, rng).reshape(nc, 9))
    t.set_porosity_values(rng.uniform(0.05, 0.35, nc))
    m = rng.uniform(0.2, 0.6, nc)
    t.set_vangenuchten_values(m, 10.0 ** rng.uniform(-5.0, -3.0, nc))
    t.set_mualem_values(m)
    t.set_constant_residual_saturation(0.15)
    t.set_water_density_type(T_.WATER_DENSITY_CONSTANT)
    t.set_boundary_pressure_type_function(lambda x, y, zz: np.full(np.shape(x), T_.NEUMANN_BC))
    U = 101325.0 + rng.normal(0.0, 2e3, nc)
    return t, U, rng


def test_long_jacobian_rows_prisms():
    """Prisms around three high-valence vertices give Jacobian rows of more
    than 96 entries (the cell gather then stages its rows in more than 48 KB of
    shared memory); parity with the oracle as for every other mesh."""
    t, U, rng = hub_prisms()
    t.setup()
    rows = np.diff(t.rowptr)
    assert rows.max() > 96, rows.max()
    o = Oracle(t.setup_view())
    Uprev = U + rng.normal(0.0, 50.0, U.size)
    t.set_dtime(DT)
    t.presolve(Uprev)
    o.snes_presolve(Uprev, DT)
    R, J = t.snes_function_jacobian(U)
    Rr, Rm = o.snes_function(U, with_mag=True)
    Jr, Jm = o.snes_jacobian(U, with_mag=True)
    assert_close(R, Rr, Rm, R_TOL, "prisms SNES residual")
    assert_close(J, Jr, Jm, J_TOL, "prisms SNES Jacobian")


@pytest.mark.parametrize("name", ["spe10_small", "wedge"])
def test_pinned_and_pageable_host_buffers(name):
    """Caller-owned page-locked R and J (as the benchmark's end-to-end loop
    passes) receive the same bits from the host-pointer call as pageable
    arrays allocated by the binding."""
    import torch

    t, o, U, Uprev, Ut = _setup(name)
    t.set_dtime(DT)
    t.presolve(Uprev)
    R1, J1 = t.snes_function_jacobian(U)
    Rp = torch.full((t.ncells,), float("nan"), dtype=torch.float64).pin_memory()
    Jp = torch.full((t.nnz,), float("nan"), dtype=torch.float64).pin_memory()
    t.snes_function_jacobian(U, Rp.numpy(), Jp.numpy())
    assert np.array_equal(Rp.numpy(), R1)
    assert np.array_equal(Jp.numpy(), J1)


def test_device_built_transmissibility_prisms():
    """Delaunay prisms with 3-D rotated K (every vertex non-hexahedral): the
    device-built Trans equals the host's to rounding of each vertex block's
    scale, and R and J meet the parity bars against the oracle on the
    host-built setup."""
    from tdycore_gb300 import workloads as W
    import tdycore_gb300 as T_

    def make(dev):
        T_.options_clear()
        if dev:
            T_.options_insert("-tdy_mpfao_setup_on_device")
        t, U0, top, src, info = W.infiltration_prisms(600, 5, rotation="full")
        t.setup(host_only=not dev)
        t.set_source_sink_values(src, cells=top)
        return t, U0

    t, U0 = make(True)
    th, _ = make(False)
    vd, vh = t.setup_view(), th.setup_view()
    Td, Th = vd["trans"], vh["trans"]
    for v in range(vh["nverts"]):
        a, b = vh["v_trans_off"][v], vh["v_trans_off"][v + 1]
        if a < b:
            assert np.all(np.abs(Td[a:b] - Th[a:b]) <= 1e-13 * np.abs(Th[a:b]).max()), v
    rng = np.random.default_rng(6)
    U = U0 + rng.normal(0.0, 3e3, U0.size)
    Uprev = U + rng.normal(0.0, 50.0, U0.size)
    o = Oracle(vh)
    t.set_dtime(DT)
    t.presolve(Uprev)
    o.snes_presolve(Uprev, DT)
    R, J = t.snes_function_jacobian(U)
    Rr, Rm = o.snes_function(U, with_mag=True)
    Jr, Jm = o.snes_jacobian(U, with_mag=True)
    assert_close(R, Rr, Rm, R_TOL, "prisms SNES residual, device-built Trans")
    rowmax = np.maximum.reduceat(Jm, t.rowptr[:-1])
    row_of = np.repeat(np.arange(t.ncells), np.diff(t.rowptr))
    assert_close(J, Jr, np.maximum(Jm, 1e-16 * rowmax[row_of]), J_TOL, "prisms SNES Jacobian, device-built Trans")
