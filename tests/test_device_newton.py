"""Device-resident backward-Euler Newton solve (TDyBackwardEulerStepDevice).

Every result is checked against the FP64 oracle: the oracle's SNES residual at
the returned state, relative to its residual at the start of the step, must
meet the requested tolerance, whether the Jacobian and inner solve ran in FP32
or FP64.  Batched instances must give each instance the same bits as solving
it alone, and the host-driven Newton (PETSc defaults, direct solve) must
agree with the device solve.
"""
import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300 import driver as D
from tdycore_gb300.workloads import batched_columns, box_column
from oracle import Oracle

pytestmark = pytest.mark.gpu

DT = 3600.0
RTOL = 1e-8


def oracle_rel_residual(t, Un, Unew, block=None):
    o = Oracle(t.setup_view())
    o.snes_presolve(Un, DT)
    F0, F1 = o.snes_function(Un), o.snes_function(Unew)
    if block is None:
        return np.linalg.norm(F1) / np.linalg.norm(F0)
    c0, c1 = block
    return np.linalg.norm(F1[c0:c1]) / np.linalg.norm(F0[c0:c1])


def oracle_meets_tolerance(t, Un, Unew, block):
    """||F(U_new)|| <= rtol ||F(U_n)|| for the instance, or, for an instance
    that starts so close to equilibrium that this is below FP64 resolution
    (the solver's step test then ends it), ||F(U_new)|| within 1e-11 of the
    residual's own error scale (the oracle's sum of term magnitudes)."""
    o = Oracle(t.setup_view())
    o.snes_presolve(Un, DT)
    c0, c1 = block
    F0 = o.snes_function(Un)[c0:c1]
    F1, M1 = o.snes_function(Unew, with_mag=True)
    F1, M1 = F1[c0:c1], M1[c0:c1]
    return (np.linalg.norm(F1) <= 1.01 * RTOL * np.linalg.norm(F0)) or (np.linalg.norm(F1) <= 1e-11 * np.linalg.norm(M1))


def column():
    T.options_clear()
    t = box_column(3, 2, 14, pfunc=lambda x, y, z: 99000.0)
    t.set_boundary_pressure_type_function(lambda x, y, z: np.where(np.asarray(z) > 1 - 1e-9, T.DIRICHLET_BC,
                                                                   T.NEUMANN_BC))
    return t


@pytest.mark.parametrize("fp32", [True, False])
def test_single_instance_meets_fp64_residual(fp32):
    import torch

    t = column()
    t.setup()
    zc = t.cell_centroids()[:, 2]
    Un = 101325.0 + 998.0 * 9.8068 * (0.5 - zc) + np.random.default_rng(2).normal(0, 300, t.ncells)
    dU = torch.tensor(Un, dtype=torch.float64, device="cuda")
    stats, its, rel = t.backward_euler_step_device(dU, DT, rtol=RTOL, fp32=fp32)
    Unew = dU.cpu().numpy()
    assert stats["converged"] == 1 and rel[0] <= RTOL
    assert oracle_rel_residual(t, Un, Unew) <= 1.01 * RTOL
    # the host Newton (PETSc defaults, sparse LU) reaches the same state
    o = Oracle(t.setup_view())
    o.snes_presolve(Un, DT)
    ref = D.SNESNewtonLS(rtol=1e-10).solve(o.snes_function, o.snes_jacobian, Un.copy(), t.rowptr, t.colidx)
    assert ref.reason > 0
    assert np.max(np.abs(Unew - ref.x) / np.abs(ref.x)) < 1e-7


def test_batch_equals_alone_and_meets_residual():
    import torch

    T.options_clear()
    tb, U0, info = batched_columns(12, seed_offset=3)
    tb.setup()
    dU = torch.tensor(U0, dtype=torch.float64, device="cuda")
    stats, its, rel = tb.backward_euler_step_device(dU, DT, rtol=RTOL, fp32=True)
    Ub = dU.cpu().numpy()
    # instances that start within FP64 resolution of equilibrium end by the
    # step test and are counted apart; the oracle check below covers both
    assert stats["converged"] + stats["step_converged"] == stats["ninstances"] == 12
    off = np.concatenate([[0], np.cumsum(info["instance_cells"])])
    for b in range(12):
        assert oracle_meets_tolerance(tb, U0, Ub, (off[b], off[b + 1])), (b, rel[b])
    # instances 0 and 7 alone: the same bits as in the batch
    off = np.concatenate([[0], np.cumsum(info["instance_cells"])])
    for b in (0, 7):
        t1, U1 = _single_block(tb, U0, info, b)
        t1.setup()
        d1 = torch.tensor(U1, dtype=torch.float64, device="cuda")
        s1, i1, r1 = t1.backward_euler_step_device(d1, DT, rtol=RTOL, fp32=True)
        assert np.array_equal(d1.cpu().numpy(), Ub[off[b]:off[b + 1]])
        assert i1[0] == its[b]


def _single_block(tb, U0, info, b):
    """Block b of a batched_columns handle as a handle of its own."""
    import tdycore_gb300.workloads as W

    blocks, props = tb._blocks, tb._props
    off = np.concatenate([[0], np.cumsum(info["instance_cells"])])
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
    t.set_boundary_pressure_type_function(lambda x, y, z: np.where(np.asarray(z) > ztop - 1e-9, T.DIRICHLET_BC,
                                                                   T.NEUMANN_BC))
    ptop = W.PREF + 998.0 * W.GRAVITY * (0.6 * ztop - ztop) + 2000.0
    t.set_boundary_pressure_function(lambda x, y, z: np.full(np.shape(x), ptop))
    return t, U0[c0:c1]


def test_cluster_preconditioner_on_prisms():
    """Delaunay prisms with per-cell anisotropic K (82 k cells, a 600 s step):
    BiCGStab preconditioned with exact solves of strong-coupling clusters
    converges the step, meets the FP64 oracle's tolerance and repeats to the
    bit."""
    import torch

    from tdycore_gb300.workloads import infiltration_prisms

    dt = 600.0
    T.options_clear()
    t, U0, top, src, info = infiltration_prisms(2000, 40)
    t.setup()
    t.set_source_sink_values(src, cells=top)
    d = torch.tensor(U0, dtype=torch.float64, device="cuda")
    stats, its, rel = t.backward_euler_step_device(d, dt, rtol=RTOL, precond="clusters")
    assert stats["converged"] == 1, (stats, rel)
    # the clusters were used (not the line fallback) and factored
    assert stats["precond_used"] == T.PRECOND_CLUSTERS and stats["clusters"] > 0, stats
    assert stats["cluster_cells"] >= 2 * stats["clusters"]
    U1 = d.cpu().numpy()
    o = Oracle(t.setup_view())
    o.snes_presolve(U0, dt)
    F0 = np.linalg.norm(o.snes_function(U0))
    F1, M1 = o.snes_function(U1, with_mag=True)
    assert np.linalg.norm(F1) <= 1.01 * RTOL * F0 or np.linalg.norm(F1) <= 1e-11 * np.linalg.norm(M1)
    d2 = torch.tensor(U0, dtype=torch.float64, device="cuda")
    t.backward_euler_step_device(d2, dt, rtol=RTOL, precond="clusters")
    assert np.array_equal(d2.cpu().numpy(), U1)


def test_cluster_factors_are_an_exact_inverse():
    """With every coupling strong (threshold 1e-300) a 54-cell column is one
    cluster, so its LU is the whole Jacobian's and the preconditioned FP64
    system is the identity: BiCGStab ends after one iteration at every Newton
    iteration, and the step equals the line-preconditioned one."""
    import torch

    def make():
        T.options_clear()
        t = box_column(3, 2, 9, pfunc=lambda x, y, z: 99000.0)
        t.set_boundary_pressure_type_function(
            lambda x, y, z: np.where(np.asarray(z) > 1 - 1e-9, T.DIRICHLET_BC, T.NEUMANN_BC))
        t.setup()
        return t

    t = make()
    assert t.ncells == 54
    zc = t.cell_centroids()[:, 2]
    Un = 101325.0 + 998.0 * 9.8068 * (0.5 - zc) + np.random.default_rng(4).normal(0, 300, t.ncells)
    d = torch.tensor(Un, dtype=torch.float64, device="cuda")
    st, its, rel = t.backward_euler_step_device(d, DT, rtol=RTOL, fp32=False, precond="clusters",
                                                cluster_threshold=1e-300)
    assert st["converged"] == 1, st
    assert st["precond_used"] == T.PRECOND_CLUSTERS and st["clusters"] == 1 and st["cluster_cells"] == 54, st
    assert st["cluster_cells_diagonal"] == 0
    assert st["linear_iterations"] == its[0] >= 1, (st, its)
    t2 = make()
    d2 = torch.tensor(Un, dtype=torch.float64, device="cuda")
    st2, _, _ = t2.backward_euler_step_device(d2, DT, rtol=RTOL, fp32=False, precond="lines")
    assert st2["converged"] == 1 and st2["precond_used"] == T.PRECOND_LINES
    U1, U2 = d.cpu().numpy(), d2.cpu().numpy()
    assert np.max(np.abs(U1 - U2) / np.abs(U2)) < 1e-9
    assert oracle_rel_residual(t, Un, U1) <= 1.01 * RTOL


@pytest.mark.parametrize("fp32", [True, False])
def test_tile_and_block_schedules_give_the_same_bits(fp32):
    """The inner solve's tile schedule (batch-wide kernels, one iteration a
    graph) and block schedule (one CTA per instance) perform the same
    operations in the same order: every instance gets the same bits, the
    same Newton and inner iteration counts, from either, and from the
    autotuned split."""
    import torch

    T.options_clear()
    tb, U0, info = batched_columns(24, seed_offset=5)
    tb.setup()
    out = {}
    for sched in ("tile", "block", "auto"):
        d = torch.tensor(U0, dtype=torch.float64, device="cuda")
        st, its, rel = tb.backward_euler_step_device(d, DT, rtol=RTOL, fp32=fp32, schedule=sched)
        out[sched] = (d.cpu().numpy(), its.copy(), st)
    assert out["block"][2]["block_instances"] == 24 and out["tile"][2]["block_instances"] == 0
    for sched in ("block", "auto"):
        assert np.array_equal(out[sched][0], out["tile"][0]), sched
        assert np.array_equal(out[sched][1], out["tile"][1]), sched
        assert out[sched][2]["linear_iterations"] == out["tile"][2]["linear_iterations"], sched
    assert out["tile"][2]["converged"] + out["tile"][2]["step_converged"] == 24


@pytest.mark.parametrize("fp32", [True, False])
def test_spmv_threads_per_row_give_the_same_bits(fp32):
    """The inner solve's sparse products sum each row in 8 phases added by a
    fixed tree whatever the threads per row: 1, 2, 4 and 8 threads, on the
    tile and the block schedule, give every instance the same bits and the
    same iteration counts (so the timed choice, kept per process, never
    changes a result)."""
    import torch

    T.options_clear()
    tb, U0, info = batched_columns(24, seed_offset=9)
    tb.setup()
    ref = None
    for sched in ("tile", "block"):
        for tpr in (1, 2, 4, 8):
            d = torch.tensor(U0, dtype=torch.float64, device="cuda")
            st, its, rel = tb.backward_euler_step_device(d, DT, rtol=RTOL, fp32=fp32, schedule=sched,
                                                         spmv_threads=tpr)
            got = (d.cpu().numpy(), its.copy(), st["linear_iterations"])
            if ref is None:
                ref = got
                continue
            assert np.array_equal(got[0], ref[0]), (sched, tpr)
            assert np.array_equal(got[1], ref[1]) and got[2] == ref[2], (sched, tpr)
