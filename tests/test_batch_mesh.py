"""A batch of independent instances as one handle (TDySetExtrudedMeshes):
block-diagonal pattern, and each block's residual/Jacobian rows equal to
those of the instance set up alone; on the GPU, the one-CTA-per-instance
evaluation gives the three-stage launches' bits."""
import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300 import workloads as W
from tdycore_gb300.workloads import layered_z, structured_surface
from oracle import Oracle


def instance(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    xy, quads = structured_surface(nx, ny, nx * 1.0, ny * 1.5, 0.1, rng)
    z = layered_z(xy.shape[0], nz, nz * 0.3, 0.1, np.random.default_rng(seed + 1))
    return xy, quads, z


def props(nc, seed):
    r = np.random.default_rng(seed)
    K = np.zeros((nc, 9))
    kh = 10.0 ** r.normal(-12, 1, nc)
    K[:, 0] = K[:, 4] = kh
    K[:, 8] = 0.3 * kh
    return K, r.uniform(0.1, 0.4, nc), 10 ** r.uniform(-5, -3, nc), r.uniform(0.2, 0.6, nc)


def configure(t, K, poro, alpha, m):
    t.set_from_options()
    t.set_permeability_values(K)
    t.set_porosity_values(poro)
    t.set_vangenuchten_values(m, alpha)
    t.set_mualem_values(m)
    t.set_water_density_type(T.WATER_DENSITY_EXPONENTIAL)
    t.set_boundary_pressure_function(lambda x, y, z: 101325.0 + 500.0 * np.sin(x + y) - 9800.0 * z)


def test_batch_blocks_match_instances():
    shapes = [(2, 3, 5), (1, 1, 7), (3, 2, 4)]
    blocks = [instance(*s, seed=10 * i) for i, s in enumerate(shapes)]
    ncs = [nx * ny * nz for nx, ny, nz in shapes]
    P = [props(n, 100 + i) for i, n in enumerate(ncs)]
    T.options_clear()
    tb = T.create_richards_mpfao()
    tb.set_extruded_meshes(blocks)
    configure(tb, *[np.concatenate([p[k] for p in P]) for k in range(4)])
    tb.setup(host_only=True)
    assert tb.ncells == sum(ncs) and list(tb.block_cells) == [0] + list(np.cumsum(ncs))
    ob = Oracle(tb.setup_view())
    rng = np.random.default_rng(5)
    U = 101325.0 + rng.normal(0, 2e4, tb.ncells)
    Up = U + rng.normal(0, 500, tb.ncells)
    ob.snes_presolve(Up, 900.0)
    R, J = ob.snes_function(U), ob.snes_jacobian(U)
    for b, (blk, p) in enumerate(zip(blocks, P)):
        c0, c1 = tb.block_cells[b], tb.block_cells[b + 1]
        # no coupling between blocks
        for i in range(c0, c1):
            cols = tb.colidx[tb.rowptr[i]:tb.rowptr[i + 1]]
            assert cols.min() >= c0 and cols.max() < c1
        T.options_clear()
        t1 = T.create_richards_mpfao()
        t1.set_extruded_mesh(*blk)
        configure(t1, *p)
        t1.setup(host_only=True)
        o1 = Oracle(t1.setup_view())
        o1.snes_presolve(Up[c0:c1], 900.0)
        assert np.array_equal(o1.snes_function(U[c0:c1]), R[c0:c1])
        assert np.array_equal(o1.snes_jacobian(U[c0:c1]), J[tb.rowptr[c0]:tb.rowptr[c1]])
        assert np.array_equal(t1.colidx + c0, tb.colidx[tb.rowptr[c0]:tb.rowptr[c1]])


@pytest.mark.gpu
def test_instance_schedule_gives_the_three_stage_bits():
    """One CTA per instance (TDyMPFAOSNESFunctionJacobianDeviceInstances)
    gives every listed instance the bits of the three-stage launches, and
    leaves the other instances' rows untouched."""
    import torch

    T.options_clear()
    tb, U0, info = W.batched_columns(40, seed_offset=9)
    tb.setup()
    tb.set_dtime(3600.0)
    dev = torch.device("cuda")
    dU = torch.tensor(U0 + np.random.default_rng(1).normal(0.0, 500.0, U0.size), dtype=torch.float64, device=dev)
    tb.presolve_device(torch.tensor(U0, dtype=torch.float64, device=dev))
    R0 = torch.empty(tb.ncells, dtype=torch.float64, device=dev)
    J0 = torch.empty(tb.nnz, dtype=torch.float64, device=dev)
    tb.snes_function_jacobian_device(dU, R0, J0)
    R1 = torch.full_like(R0, float("nan"))
    J1 = torch.full_like(J0, float("nan"))
    tb.snes_function_jacobian_device_instances(dU, R1, J1, list(range(40)))
    torch.cuda.synchronize()
    assert torch.equal(R0, R1) and torch.equal(J0, J1)
    # a subset: listed rows recomputed bit for bit, the others left as they were
    off = np.concatenate([[0], np.cumsum(info["instance_cells"])])
    R2 = torch.full_like(R0, 7.0)
    J2 = torch.full_like(J0, 7.0)
    pick = [3, 17, 39]
    tb.snes_function_jacobian_device_instances(dU, R2, J2, pick)
    torch.cuda.synchronize()
    R0h, R2h = R0.cpu().numpy(), R2.cpu().numpy()
    J0h, J2h = J0.cpu().numpy(), J2.cpu().numpy()
    mask = np.zeros(tb.ncells, bool)
    for g in pick:
        mask[off[g]:off[g + 1]] = True
    assert np.array_equal(R2h[mask], R0h[mask]) and np.all(R2h[~mask] == 7.0)
    rows = np.repeat(mask, np.diff(tb.rowptr))
    assert np.array_equal(J2h[rows], J0h[rows]) and np.all(J2h[~rows] == 7.0)
