"""Seeded synthetic workloads for the MPFA-O Richards path.

Each builder returns a configured (not yet set up) :class:`tdycore_gb300.TDy`
together with the pressure state to evaluate.  Fields are drawn from seeded
generators so every run, test and benchmark sees the same inputs.

* ``box_column``      -- the reference's regression geometries
  (demo/transient/transient_snes_mpfaof90.F90, transient_mpfaof90.F90).
* ``hydrostatic_box`` -- 10x10x10 cells over a 1 m cube, k = 1e-11 m^2,
  porosity 0.25, van Genuchten alpha = 1e-4 Pa^-1, m = 0.3, Sr = 0.15,
  hydrostatic pressure with 101325 Pa at the top face, rho = 998.2 kg/m^3
  (the density constant of this workload; the reference's constant-density
  EOS uses 998.0), Dirichlet on the top face and no flow elsewhere.
* ``spe10_like``      -- 60x220x85 hexahedra over 365.76 x 670.56 x 51.816 m
  (the SPE10 model-2 grid) with vertices jittered by up to 10% of the cell
  size (x, y per vertical vertex line, z per vertex), log10 k ~ N(-13, 1.5^2)
  smoothed by a 5-cell Gaussian kernel and re-standardised, kz = 0.1 kh,
  porosity ~ U(0.05, 0.35), alpha ~ logU(1e-5, 1e-3), m ~ U(0.2, 0.6) per
  cell, and hydrostatic pressure plus N(0, 5e3 Pa) noise.  A seeded
  synthetic field stands in for the SPE10 permeability data.
* ``wedge_extruded``  -- a seeded Delaunay triangulation extruded into
  layers (prisms), full-tensor permeability with random rotations.
"""
from __future__ import annotations

import numpy as np

from . import (DIRICHLET_BC, NEUMANN_BC, WATER_DENSITY_CONSTANT, WATER_DENSITY_EXPONENTIAL, TDy,
               create_richards_mpfao)

MASTER_SEED = 20261203
GRAVITY = 9.8068
PREF = 101325.0


def _rng(sub: int) -> np.random.Generator:
    return np.random.default_rng([MASTER_SEED, sub])


def structured_surface(nx, ny, lx, ly, jitter=0.0, rng=None):
    """Surface vertices (x fastest) and counter-clockwise quads of an nx*ny grid."""
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    if jitter > 0.0:
        dx, dy = lx / nx, ly / ny
        jx = rng.uniform(-jitter, jitter, X.shape) * dx
        jy = rng.uniform(-jitter, jitter, Y.shape) * dy
        jx[:, 0] = jx[:, -1] = 0.0
        jy[0, :] = jy[-1, :] = 0.0
        X = X + jx
        Y = Y + jy
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    v0 = (j * (nx + 1) + i).ravel()
    quads = np.stack([v0, v0 + 1, v0 + nx + 2, v0 + nx + 1], axis=1).astype(np.int32)
    return xy, quads


def layered_z(nv2, nz, lz, jitter=0.0, rng=None, ztop=None):
    """Vertex elevations per level (level-major), optional per-vertex jitter."""
    levels = np.linspace(0.0, lz, nz + 1)
    z = np.repeat(levels[:, None], nv2, axis=1)
    if jitter > 0.0:
        dz = lz / nz
        jz = rng.uniform(-jitter, jitter, z.shape) * dz
        jz[0, :] = jz[-1, :] = 0.0
        z = z + jz
    return z


def hydrostatic(zc, ztop, rho, g=GRAVITY, ptop=PREF):
    return ptop + rho * g * (ztop - zc)


def box_column(nx, ny, nz, *, density=WATER_DENSITY_EXPONENTIAL, gmatrix=0, bc_type=None, pfunc=None,
               perm=1e-10, porosity=0.115, sr=0.115) -> TDy:
    """The reference's transient regression geometry on [0,1]^3."""
    t = create_richards_mpfao()
    t.set_box_mesh(nx, ny, nz)
    t.set_from_options()
    t.set_constant_tensor_permeability([perm, 0, 0, 0, perm, 0, 0, 0, perm])
    t.set_constant_residual_saturation(sr)
    t.set_constant_porosity(porosity)
    t.set_water_density_type(density)
    t.set_gmatrix_method(gmatrix)
    if bc_type is not None:
        t.set_boundary_condition_type(bc_type)
    if pfunc is not None:
        t.set_boundary_pressure_function(pfunc)
    return t


def top_dirichlet_types(ztop, tol=1e-9):
    return lambda x, y, z: np.where(np.asarray(z) > ztop - tol, DIRICHLET_BC, NEUMANN_BC)


def hydrostatic_box(n=10, rho=998.2):
    """10x10x10 box workload; returns (tdy, U0, info)."""
    t = create_richards_mpfao()
    t.set_box_mesh(n, n, n)
    t.set_from_options()
    t.set_constant_isotropic_permeability(1e-11)
    t.set_constant_porosity(0.25)
    t.set_constant_residual_saturation(0.15)
    nc = n ** 3
    t.set_vangenuchten_values(np.full(nc, 0.3), np.full(nc, 1e-4))
    t.set_mualem_values(np.full(nc, 0.3))
    t.set_water_density_type(WATER_DENSITY_CONSTANT)
    t.set_boundary_pressure_type_function(top_dirichlet_types(1.0))
    t.set_boundary_pressure_function(lambda x, y, z: PREF)
    k = np.arange(nc) // (n * n)
    zc = (k + 0.5) / n
    U0 = hydrostatic(zc, 1.0, rho)
    return t, U0, {"workload": f"hydrostatic_box_{n}x{n}x{n}", "ncells": nc, "rho": rho}


def _correlated_log10k(shape, rng, mean=-13.0, std=1.5, sigma=5.0):
    from scipy.ndimage import gaussian_filter

    g = rng.standard_normal(shape)
    g = gaussian_filter(g, sigma=sigma, mode="reflect")
    g = (g - g.mean()) / g.std()
    return mean + std * g


def spe10_like(nx=60, ny=220, nz=85, lx=365.76, ly=670.56, lz=51.816, jitter=0.10, seed_offset=0):
    """The 60x220x85 jittered hex workload; returns (tdy, U, info)."""
    rng = _rng(1 + seed_offset)
    xy, quads = structured_surface(nx, ny, lx, ly, jitter, rng)
    z = layered_z(xy.shape[0], nz, lz, jitter, _rng(2 + seed_offset))
    t = create_richards_mpfao()
    t.set_extruded_mesh(xy, quads, z)
    t.set_from_options()
    nc = nx * ny * nz
    log10k = _correlated_log10k((nz, ny, nx), _rng(3 + seed_offset)).ravel()
    kh = 10.0 ** log10k
    K = np.zeros((nc, 9))
    K[:, 0] = kh
    K[:, 4] = kh
    K[:, 8] = 0.1 * kh
    t.set_permeability_values(K)
    r = _rng(4 + seed_offset)
    t.set_porosity_values(r.uniform(0.05, 0.35, nc))
    alpha = 10.0 ** r.uniform(-5.0, -3.0, nc)
    m = r.uniform(0.2, 0.6, nc)
    t.set_vangenuchten_values(m, alpha)
    t.set_mualem_values(m)
    t.set_constant_residual_saturation(0.15)
    t.set_water_density_type(WATER_DENSITY_CONSTANT)
    t.set_boundary_pressure_type_function(top_dirichlet_types(lz))
    t.set_boundary_pressure_function(lambda x, y, zz: PREF)
    # cell-centre elevations: mean of the 8 vertex elevations
    zl = z.reshape(nz + 1, ny + 1, nx + 1)
    zc = 0.125 * (zl[:-1, :-1, :-1] + zl[:-1, :-1, 1:] + zl[:-1, 1:, :-1] + zl[:-1, 1:, 1:] +
                  zl[1:, :-1, :-1] + zl[1:, :-1, 1:] + zl[1:, 1:, :-1] + zl[1:, 1:, 1:]).ravel()
    U = hydrostatic(zc, lz, 998.0) + _rng(5 + seed_offset).normal(0.0, 5e3, nc)
    info = {"workload": f"spe10_like_hex_{nx}x{ny}x{nz}_jitter{jitter}", "ncells": nc, "seed": MASTER_SEED,
            "grid": [nx, ny, nz], "extent_m": [lx, ly, lz]}
    return t, U, info


def delaunay_surface(npts, lx, ly, rng):
    """Delaunay triangulation (counter-clockwise triangles) of ``npts``
    uniform random points in [0, lx] x [0, ly] plus points along the four
    sides at the mean interior spacing h (corners included); random points
    closer than h/4 to a side are dropped.  Without the side points every
    side is one hull edge, and interior points close to it form triangles
    with angles near 180 degrees, on which MPFA-O is far from monotone
    (negative Jacobian diagonals, indefinite linear systems)."""
    from scipy.spatial import Delaunay

    pts = rng.uniform(0.0, 1.0, (npts, 2)) * [lx, ly]
    h = np.sqrt(lx * ly / max(npts, 1))
    margin = np.minimum(np.minimum(pts[:, 0], lx - pts[:, 0]), np.minimum(pts[:, 1], ly - pts[:, 1]))
    pts = pts[margin >= 0.25 * h]
    nx, ny = max(int(round(lx / h)), 1), max(int(round(ly / h)), 1)
    sx, sy = np.linspace(0.0, lx, nx + 1), np.linspace(0.0, ly, ny + 1)
    side = np.vstack([np.c_[sx, np.zeros_like(sx)], np.c_[sx, np.full_like(sx, ly)],
                      np.c_[np.zeros(ny - 1), sy[1:-1]], np.c_[np.full(ny - 1, lx), sy[1:-1]]])
    pts = np.vstack([side, pts])
    tri = Delaunay(pts)
    simp = tri.simplices.astype(np.int32)
    # counter-clockwise orientation
    a, b, c = pts[simp[:, 0]], pts[simp[:, 1]], pts[simp[:, 2]]
    cross = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    flip = cross < 0
    simp[flip] = simp[flip][:, [0, 2, 1]]
    # drop degenerate triangles (collinear side points)
    area = 0.5 * np.abs(cross)
    keep = area > 1e-9 * lx * ly / max(len(simp), 1)
    return pts, simp[keep]


def random_spd(nc, rng, mean=-12.0, std=1.0, rotation="full", anisotropy_std=None):
    """Per-cell symmetric positive-definite K with log10 eigenvalues ~ N(mean,
    std) and a random rotation: a uniform random 3-D rotation ("full") or a
    rotation by a uniform angle about the vertical axis ("vertical", which
    leaves K_xz = K_yz = 0 and the horizontal 2x2 block full).  With
    ``anisotropy_std`` s the three log10 eigenvalues of a cell share a common
    N(0, std^2 - s^2) part and differ by independent N(0, s^2) parts (each
    eigenvalue still ~ N(mean, std^2); log10 of the anisotropy ratio then has
    standard deviation s * sqrt(2) instead of std * sqrt(2))."""
    if anisotropy_std is None:
        eig = 10.0 ** (mean + std * rng.standard_normal((nc, 3)))
    else:
        if not 0.0 <= anisotropy_std <= std:
            raise ValueError("anisotropy_std must lie in [0, std]")
        common = np.sqrt(std * std - anisotropy_std * anisotropy_std) * rng.standard_normal((nc, 1))
        eig = 10.0 ** (mean + common + anisotropy_std * rng.standard_normal((nc, 3)))
    if rotation == "full":
        q, _ = np.linalg.qr(rng.standard_normal((nc, 3, 3)))
    elif rotation == "vertical":
        th = rng.uniform(0.0, 2.0 * np.pi, nc)
        c, s = np.cos(th), np.sin(th)
        q = np.zeros((nc, 3, 3))
        q[:, 0, 0], q[:, 0, 1], q[:, 1, 0], q[:, 1, 1], q[:, 2, 2] = c, -s, s, c, 1.0
    else:
        raise ValueError(f"rotation must be 'full' or 'vertical', not {rotation!r}")
    K = np.einsum("nij,nj,nkj->nik", q, eig, q)
    return 0.5 * (K + np.transpose(K, (0, 2, 1)))


def wedge_extruded(npts=200, nlayers=4, lx=1000.0, ly=1000.0, seed_offset=0, dz_range=(0.1, 2.0)):
    """Extruded Delaunay prisms with full-tensor K; returns (tdy, U, info)."""
    rng = _rng(10 + seed_offset)
    xy, tris = delaunay_surface(npts, lx, ly, rng)
    dz = rng.uniform(*dz_range, nlayers)
    levels = np.concatenate([[0.0], np.cumsum(dz)])
    z = np.repeat(levels[:, None], xy.shape[0], axis=1)
    t = create_richards_mpfao()
    t.set_extruded_mesh(xy, tris, z)
    t.set_from_options()
    nc = nlayers * tris.shape[0]
    t.set_permeability_values(random_spd(nc, _rng(11 + seed_offset)).reshape(nc, 9))
    r = _rng(12 + seed_offset)
    t.set_porosity_values(r.uniform(0.05, 0.35, nc))
    m = r.uniform(0.2, 0.6, nc)
    t.set_vangenuchten_values(m, 10.0 ** r.uniform(-5.0, -3.0, nc))
    t.set_mualem_values(m)
    t.set_water_density_type(WATER_DENSITY_EXPONENTIAL)
    ztop = levels[-1]
    t.set_boundary_pressure_type_function(top_dirichlet_types(ztop))
    t.set_boundary_pressure_function(lambda x, y, zz: PREF - 2e3)
    layer = np.arange(nc) // tris.shape[0]
    zc = 0.5 * (levels[layer] + levels[layer + 1])
    U = hydrostatic(zc, ztop, 998.0) + _rng(13 + seed_offset).normal(0.0, 3e3, nc)
    return t, U, {"workload": f"wedge_{tris.shape[0]}tri_{nlayers}layers", "ncells": nc}


def batched_columns(ninst=4096, seed_offset=0, cell=1.0, gap=1.0, top_excess=2000.0):
    """Independent hexahedral subdomains in one handle (TDySetExtrudedMeshes):
    nx, ny ~ U{1..8}, nz ~ U{10..100}, layer thickness ~ U(0.05, 0.5) m per
    instance, horizontal cells of ``cell`` m; per instance a homogeneous
    isotropic k (log10 ~ N(-12, 1) m^2), porosity ~ U(0.05, 0.35), van
    Genuchten alpha ~ logU(1e-5, 1e-3) 1/Pa and m ~ U(0.2, 0.6), Sr 0.15.
    Instances sit side by side along x (``gap`` m apart).  Start: hydrostatic
    (rho 998 kg/m^3) with the water table at 40 % of the depth from the top,
    plus N(0, 10 Pa) noise;
    boundary: on each instance's top face Dirichlet at its hydrostatic
    pressure plus ``top_excess`` Pa (infiltration), no flow elsewhere.
    Returns (tdy, U0, info)."""
    r = _rng(20 + seed_offset)
    nx = r.integers(1, 9, ninst)
    ny = r.integers(1, 9, ninst)
    nz = r.integers(10, 101, ninst)
    dz = r.uniform(0.05, 0.5, ninst)
    blocks, x0 = [], 0.0
    xs, ztops = [], []
    for b in range(ninst):
        xy, quads = structured_surface(int(nx[b]), int(ny[b]), cell * nx[b], cell * ny[b])
        xy[:, 0] += x0
        xs.append(x0)
        x0 += cell * nx[b] + gap
        depth = dz[b] * nz[b]
        z = layered_z(xy.shape[0], int(nz[b]), depth)
        ztops.append(depth)
        blocks.append((xy, quads, z))
    ncell = (nx * ny * nz).astype(np.int64)
    t = create_richards_mpfao()
    t.set_extruded_meshes(blocks)
    t.set_from_options()
    rp = _rng(21 + seed_offset)
    k = np.repeat(10.0 ** rp.normal(-12.0, 1.0, ninst), ncell)
    K = np.zeros((k.size, 9))
    K[:, 0] = K[:, 4] = K[:, 8] = k
    t.set_permeability_values(K)
    poro = np.repeat(rp.uniform(0.05, 0.35, ninst), ncell)
    t.set_porosity_values(poro)
    m = np.repeat(rp.uniform(0.2, 0.6, ninst), ncell)
    alpha = np.repeat(10.0 ** rp.uniform(-5.0, -3.0, ninst), ncell)
    t.set_vangenuchten_values(m, alpha)
    t.set_mualem_values(m)
    t.set_constant_residual_saturation(0.15)
    t.set_water_density_type(WATER_DENSITY_CONSTANT)
    xs, ztops = np.asarray(xs), np.asarray(ztops)

    def which(x):
        # instance of a boundary face by its x: split at the middle of the gaps
        # (a face centroid on an instance's edge may round to either side of it)
        return np.clip(np.searchsorted(xs - 0.5 * gap, np.asarray(x), side="right") - 1, 0, ninst - 1)

    t.set_boundary_pressure_type_function(
        lambda x, y, z: np.where(np.asarray(z) > ztops[which(x)] - 1e-9, DIRICHLET_BC, NEUMANN_BC))
    ptop = PREF + 998.0 * GRAVITY * (0.6 * ztops - ztops) + top_excess
    t.set_boundary_pressure_function(lambda x, y, z: ptop[which(x)])
    # cell-centre depths: layer centres of each instance
    U = np.empty(int(ncell.sum()))
    o = 0
    for b in range(ninst):
        kk = np.arange(int(nz[b]))
        zc = (kk + 0.5) * dz[b]
        depth = dz[b] * nz[b]
        table = 0.6 * depth
        p = PREF + 998.0 * GRAVITY * (table - zc)
        U[o:o + ncell[b]] = np.repeat(p, nx[b] * ny[b])
        o += ncell[b]
    # 10 Pa of noise: an exactly hydrostatic state puts every vertical face at
    # an upwinding tie (T.P + rho G = 0 up to rounding)
    U += _rng(22 + seed_offset).normal(0.0, 10.0, U.size)
    info = {"workload": f"batched_columns_{ninst}", "ninstances": ninst, "ncells": int(ncell.sum()),
            "seed": MASTER_SEED, "instance_cells": ncell}
    # the inputs, for building one instance on its own
    t._blocks = blocks
    t._props = {"K": K, "poro": poro, "m": m, "alpha": alpha}
    return t, U, info


def infiltration_prisms(ntri=200_000, nlayers=40, lx=1000.0, ly=1000.0, seed_offset=0, top_flux=1e-7,
                        rotation="vertical", suction=2.0e4, vg_alpha=1.0e-4, vg_m=0.5, anisotropy_std=None):
    """Infiltration into a dry soil on triangular prisms: a seeded Delaunay
    triangulation of uniform random points on an lx x ly square (about
    ``ntri`` triangles), extruded into ``nlayers`` z-aligned layers of
    thickness ~ U(0.1, 2) m.  Per cell a symmetric positive-definite K with
    log10 eigenvalues ~ N(-12, 1) and a random rotation (``rotation``, see
    random_spd) and porosity ~ U(0.05, 0.35); one van Genuchten/Mualem soil
    (``vg_alpha`` 1/Pa, ``vg_m``), Sr 0.15, constant density.  Start: uniform
    pressure Pref - ``suction``.  Boundaries: no flow; the infiltration
    (``top_flux`` m/s downward through the top surface) is a source
    rho * q * A in each top cell.

    Why these choices (measured with the oracle and an exact or Krylov linear
    solve on 5 k - 8 M cells):
    * rotations about the vertical axis: with a random 3-D rotation the
      two-point gravity term of the reference (src/fv/mpfao/tdympfao.c:
      2145-2265, A (n . K u) (g . u) with u the centroid-to-centroid
      direction, zero on the vertical faces of z-aligned prisms) cannot
      balance the MPFA-O pressure flux n . K grad(p) that K_xz and K_yz carry
      on those faces; no hydrostatic or uniform start is near the discrete
      equilibrium and Newton stalls at 1e-2 to 1e-3 relative residual;
    * one soil: with van Genuchten parameters that differ between neighbours
      (per cell or per layer), upwinded kr jumps wherever a flux passes
      through zero, the residual has first-order kinks there and Newton's
      line search stalls at 1e-4 to 1e-2; with one soil the jump is of second
      order and Newton converges quadratically (3-6 iterations per step).

    Returns (tdy, U0, top_cells, top_source, info)."""
    rng = _rng(30 + seed_offset)
    xy, tris = delaunay_surface(max(ntri // 2, 3), lx, ly, rng)
    dz = rng.uniform(0.1, 2.0, nlayers)
    levels = np.concatenate([[0.0], np.cumsum(dz)])
    z = np.repeat(levels[:, None], xy.shape[0], axis=1)
    t = create_richards_mpfao()
    t.set_extruded_mesh(xy, tris, z)
    t.set_from_options()
    nt = tris.shape[0]
    nc = nlayers * nt
    K = random_spd(nc, _rng(31 + seed_offset), rotation=rotation, anisotropy_std=anisotropy_std)
    t.set_permeability_values(K.reshape(nc, 9))
    r = _rng(32 + seed_offset)
    t.set_porosity_values(r.uniform(0.05, 0.35, nc))
    m = np.full(nc, vg_m)
    t.set_vangenuchten_values(m, np.full(nc, vg_alpha))
    t.set_mualem_values(m)
    t.set_constant_residual_saturation(0.15)
    t.set_water_density_type(WATER_DENSITY_CONSTANT)
    t.set_boundary_pressure_type_function(lambda x, y, zz: np.full(np.shape(x), NEUMANN_BC))
    U = np.full(nc, PREF - suction)
    a, b, c = xy[tris[:, 0]], xy[tris[:, 1]], xy[tris[:, 2]]
    area = 0.5 * np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
    top = np.arange((nlayers - 1) * nt, nc, dtype=np.int32)
    info = {"workload": f"infiltration_prisms_{nt}tri_{nlayers}layers", "ncells": nc, "seed": MASTER_SEED,
            "top_flux_m_per_s": top_flux, "rotation": rotation, "initial_pressure_pa": PREF - suction,
            "van_genuchten": {"alpha_per_pa": vg_alpha, "m": vg_m}, "depth_m": float(levels[-1])}
    return t, U, top, 998.0 * top_flux * area, info

