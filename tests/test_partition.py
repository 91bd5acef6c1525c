"""Layer-slab partition and halo exchange (multi-rank plan of the F+J path):
the partition arithmetic in one process; a two-rank gloo run on the CPU in
which every rank evaluates its owned rows of R and J (oracle, host setup of
its local slab) after one ghost exchange, and the owned rows match the
whole-mesh evaluation; and the same two-rank run with the CUDA evaluation
(each rank sets up its slab on the device, the ghosts travel through host
buffers over gloo), whose owned rows equal the whole-mesh GPU evaluation bit
for bit.
"""
import os
import socket

import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300.partition import SlabPartition
from tdycore_gb300.workloads import layered_z, structured_surface, top_dirichlet_types

NX, NY, NZ = 4, 3, 7
LX, LY, LZ = 40.0, 30.0, 7.0
DT = 1800.0


def global_fields():
    rng = np.random.default_rng(77)
    xy, quads = structured_surface(NX, NY, LX, LY, 0.1, rng)
    z = layered_z(xy.shape[0], NZ, LZ, 0.1, np.random.default_rng(78))
    nc = NX * NY * NZ
    r = np.random.default_rng(79)
    K = np.zeros((nc, 9))
    kh = 10.0 ** r.normal(-12.0, 1.0, nc)
    K[:, 0], K[:, 4], K[:, 8] = kh, kh, 0.1 * kh
    K[:, 1] = K[:, 3] = 0.2 * kh  # full tensor in x-y
    poro = r.uniform(0.1, 0.3, nc)
    alpha = 10.0 ** r.uniform(-5.0, -3.0, nc)
    m = r.uniform(0.2, 0.6, nc)
    U = 101325.0 + r.normal(0.0, 3e4, nc)
    Uprev = U + r.normal(0.0, 1e3, nc)
    return dict(xy=xy, quads=quads, z=z, K=K, poro=poro, alpha=alpha, m=m, U=U, Uprev=Uprev)


def build(f, levels, cells, device=False):
    """Setup (host only, or host and device) of the mesh made of the given
    vertex levels, with the properties of the given global cells."""
    T.options_clear()
    t = T.create_richards_mpfao()
    t.set_extruded_mesh(f["xy"], f["quads"], f["z"][levels])
    t.set_from_options()
    t.set_permeability_values(f["K"][cells])
    t.set_porosity_values(f["poro"][cells])
    t.set_vangenuchten_values(f["m"][cells], f["alpha"][cells])
    t.set_mualem_values(f["m"][cells])
    t.set_constant_residual_saturation(0.15)
    t.set_water_density_type(T.WATER_DENSITY_EXPONENTIAL)
    t.set_boundary_pressure_type_function(top_dirichlet_types(f["z"].max()))
    t.set_boundary_pressure_function(lambda x, y, zz: 101325.0)
    t.setup(host_only=not device)
    return t


def evaluate(t, U, Uprev):
    from oracle import Oracle

    o = Oracle(t.setup_view())
    o.snes_presolve(Uprev, DT)
    R = o.snes_function(U)
    J = o.snes_jacobian(U)
    return R, J


def test_partition_arithmetic():
    ncol = NX * NY
    for P in (1, 2, 3, NZ):
        part = SlabPartition(ncol, NZ, P)
        owned = np.concatenate([part.local(r).cells[part.local(r).owned] for r in range(P)])
        assert np.array_equal(owned, np.arange(ncol * NZ)), "every cell owned exactly once"
        sizes = [part.starts[r + 1] - part.starts[r] for r in range(P)]
        assert max(sizes) - min(sizes) <= 1
        for r in range(P):
            s = part.local(r)
            # what a rank receives from a neighbour is what the neighbour sends it
            for nb, idx in s.recv.items():
                other = part.local(nb)
                assert np.array_equal(s.cells[idx], other.cells[other.send[r]])
                assert all(part.owner_of_cell(c) == nb for c in s.cells[idx])
        # lowest-owner rule for vertex levels
        for kv in range(NZ + 1):
            ks = [k for k in (kv - 1, kv) if 0 <= k < NZ]
            assert part.owner_of_vertex_level(kv) == min(part.owner_of_layer(k) for k in ks)
    with pytest.raises(ValueError):
        SlabPartition(ncol, NZ, NZ + 1)


def test_ghosts_are_the_fvm_overlap():
    """The ghost cells of a slab are exactly the non-owned columns of its
    owned rows in the Jacobian pattern (cells sharing a vertex)."""
    f = global_fields()
    ncol = NX * NY
    t = build(f, slice(0, NZ + 1), np.arange(ncol * NZ))
    part = SlabPartition(ncol, NZ, 3)
    for r in range(3):
        s = part.local(r)
        owned = s.cells[s.owned]
        cols = np.unique(np.concatenate([t.colidx[t.rowptr[i]:t.rowptr[i + 1]] for i in owned]))
        assert np.array_equal(np.setdiff1d(cols, owned), s.cells[~s.owned])


def evaluate_gpu(t, U, Uprev):
    """The CUDA evaluation through the host-pointer C-ABI."""
    t.set_dtime(DT)
    t.presolve(Uprev)
    return t.snes_function_jacobian(U)


def _rank_main(rank, world, port, out_dir, device=False):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f = global_fields()
        ncol = NX * NY
        part = SlabPartition(ncol, NZ, world)
        s = part.local(rank)
        # each rank holds only its owned values; ghosts come from the exchange
        U = np.full(s.nlocal, np.nan)
        Up = np.full(s.nlocal, np.nan)
        U[s.owned] = f["U"][s.cells[s.owned]]
        Up[s.owned] = f["Uprev"][s.cells[s.owned]]
        s.exchange(U, dist)
        s.exchange(Up, dist)
        assert np.array_equal(U, f["U"][s.cells]) and np.array_equal(Up, f["Uprev"][s.cells])
        t = build(f, s.levels(), s.cells, device=device)
        R, J = (evaluate_gpu if device else evaluate)(t, U, Up)
        rows, rp, cols, vals = s.global_rows(t.rowptr, t.colidx, J)
        t.destroy()
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), rows=rows, R=R[s.owned_local], rp=rp, cols=cols,
                 vals=vals)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _check_two_ranks(tmp_path, device):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path), device), nprocs=world, join=True)
    f = global_fields()
    ncol = NX * NY
    t = build(f, slice(0, NZ + 1), np.arange(ncol * NZ), device=device)
    R, J = (evaluate_gpu if device else evaluate)(t, f["U"], f["Uprev"])
    seen = np.zeros(t.ncells, bool)
    for r in range(world):
        d = np.load(tmp_path / f"rank{r}.npz")
        rows = d["rows"]
        assert not seen[rows].any()
        seen[rows] = True
        # owned residual rows: the same interaction regions, the same operations
        assert np.array_equal(d["R"], R[rows])
        for k, i in enumerate(rows):
            a, b = d["rp"][k], d["rp"][k + 1]
            assert np.array_equal(d["cols"][a:b], t.colidx[t.rowptr[i]:t.rowptr[i + 1]])
            assert np.array_equal(d["vals"][a:b], J[t.rowptr[i]:t.rowptr[i + 1]])
    assert seen.all()
    t.destroy()


def test_two_rank_halo_exchange_matches_whole_mesh(tmp_path):
    _check_two_ranks(tmp_path, device=False)


@pytest.mark.gpu
def test_two_rank_cuda_slabs_match_whole_mesh_gpu(tmp_path):
    """Two ranks on the one GPU (separate processes and contexts; their
    kernels never wait on each other): owned rows of the CUDA evaluation of
    each slab equal the whole-mesh CUDA evaluation bit for bit."""
    _check_two_ranks(tmp_path, device=True)
