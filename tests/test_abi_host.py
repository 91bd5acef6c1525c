"""CPU tests: C-ABI surface, call-order errors and host-side setup properties."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300 import workloads as W
from oracle import Oracle

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"^\s*(?:TDyErrorCode|const char \*)\s*(TDy\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(T.lib, n)]
    assert not missing, missing


def test_call_order_and_unsupported_paths():
    t = T.TDy()
    with pytest.raises(T.TDyError):
        t.set_discretization(T.MPFA_O)  # before TDySetMode (src/tdycore.c:839-842)
    with pytest.raises(T.TDyError) as e:
        t.set_mode(T.TH)
    assert e.value.code == 56
    t.set_mode(T.RICHARDS)
    with pytest.raises(T.TDyError):
        t.set_discretization(T.BDM)
    t.set_discretization(T.MPFA_O)
    t.set_box_mesh(2, 2, 2)
    with pytest.raises(T.TDyError):
        t.setup()  # TDySetFromOptions not called (src/tdycore.c:737-739)
    T.options_clear()
    t.set_from_options()
    t.setup(host_only=True)
    with pytest.raises(T.TDyError) as e:
        t.snes_function(np.full(8, 1e5))
    assert e.value.code == T.TDY_ERR_GPU


def test_options_database():
    T.options_clear()
    T.options_insert("-tdy_water_density EXPONENTIAL -tdy_mpfao_gmatrix_method MPFAO_GMATRIX_TPF "
                     "-tdy_mpfao_boundary_condition_type NEUMANN_BC -tdy_gravity 9.81")
    t = T.create_richards_mpfao()
    t.set_box_mesh(2, 2, 2)
    t.set_from_options()
    t.setup(host_only=True)
    v = t.setup_view()
    T.options_clear()
    assert v["rho_type"] == T.WATER_DENSITY_EXPONENTIAL
    assert v["gmatrix_method"] == T.MPFAO_GMATRIX_TPF
    assert v["bc_type"] == T.NEUMANN_BC
    assert v["gravity"] == 9.81
    T.options_insert("-tdy_water_density NOT_A_MODEL")
    t2 = T.create_richards_mpfao()
    with pytest.raises(T.TDyError):
        t2.set_from_options()
    T.options_clear()


def _host(t):
    t.setup(host_only=True)
    return t.setup_view()


def test_box_counts_and_numbering():
    T.options_clear()
    t = W.box_column(3, 4, 5)
    v = _host(t)
    assert v["ncells"] == 60 and v["nverts"] == 4 * 5 * 6
    assert v["nfaces"] == 6 * 12 + 5 * (3 * 5 + 4 * 4)
    assert v["nbnd"] == 2 * (3 * 4 + 3 * 5 + 4 * 5)
    x = t.cell_centroids()
    # x fastest, then y, then z (DMPlexCreateBoxMesh numbering)
    assert np.allclose(x[1] - x[0], [1 / 3, 0, 0]) and np.allclose(x[3] - x[0], [0, 1 / 4, 0])
    assert np.allclose(x[12] - x[0], [0, 0, 1 / 5])
    assert np.allclose(t.cell_volumes(), 1.0 / 60)


@pytest.mark.parametrize("builder", ["box", "jittered", "wedge"])
def test_pattern_matches_independent_pattern(builder):
    T.options_clear()
    if builder == "box":
        t = W.box_column(4, 3, 5)
    elif builder == "jittered":
        t, _, _ = W.spe10_like(6, 5, 4, lx=36.0, ly=15.0, lz=2.4)
    else:
        t, _, _ = W.wedge_extruded(npts=30, nlayers=3)
    v = _host(t)
    o = Oracle(v)
    rp, ci = o.pattern()
    assert np.array_equal(rp, v["rowptr"]) and np.array_equal(ci, v["colidx"])
    # interior hex rows have 27 entries, sorted and unique
    rows = np.diff(v["rowptr"])
    assert rows.max() <= 64
    for i in range(v["ncells"]):
        r = v["colidx"][v["rowptr"][i]:v["rowptr"][i + 1]]
        assert np.all(np.diff(r) > 0) and i in r
    if builder == "box":
        assert rows.max() == 27


def _linear_field_fluxes(t, grad, K):
    """Trans rows applied to an exactly linear pressure field."""
    v = _host(t)
    nc = v["ncells"]
    xc = v["centroid"].reshape(-1, 3)
    fc = v["face_centroid"].reshape(-1, 3)
    P = np.concatenate([xc @ grad, fc[v["bnd_face"]] @ grad])
    err, scale = 0.0, 0.0
    for vtx in range(v["nverts"]):
        r0, r1 = v["v_row_off"][vtx], v["v_row_off"][vtx + 1]
        c0, c1 = v["v_col_off"][vtx], v["v_col_off"][vtx + 1]
        if r1 == r0:
            continue
        T_ = v["trans"][v["v_trans_off"][vtx]:v["v_trans_off"][vtx + 1]].reshape(r1 - r0, c1 - c0)
        TP = T_ @ P[v["col_ext"][c0:c1]]
        for k, f in enumerate(v["row_face"][r0:r1]):
            n = v["face_normal"][3 * f:3 * f + 3]
            exact = v["face_area"][f] / v["face_nverts"][f] * (n @ (K @ grad))
            err = max(err, abs(TP[k] - exact))
            scale = max(scale, abs(exact))
    return err, scale


@pytest.mark.parametrize("builder", ["box", "jittered", "wedge"])
def test_mpfao_exact_for_linear_pressure(builder):
    """MPFA-O with homogeneous K reproduces linear pressure fields exactly:
    Trans . P equals A_subface * n . K grad(P) on every row (interior and
    Dirichlet boundary), on orthogonal, jittered-hex and prism meshes."""
    T.options_clear()
    K = np.array([[2e-12, 3e-13, 0.0], [3e-13, 1e-12, 1e-13], [0.0, 1e-13, 5e-13]])
    rng = np.random.default_rng(3)
    if builder == "box":
        xy, cells = W.structured_surface(3, 4, 1.0, 1.0)
        z = W.layered_z(xy.shape[0], 3, 1.0)
    elif builder == "jittered":
        xy, cells = W.structured_surface(5, 4, 30.0, 12.0, 0.1, rng)
        z = W.layered_z(xy.shape[0], 4, 2.4, 0.1, rng)
    else:
        xy, cells = W.delaunay_surface(25, 100.0, 80.0, rng)
        z = np.repeat(np.array([0.0, 0.7, 2.0])[:, None], xy.shape[0], axis=1)
    t = T.create_richards_mpfao()
    t.set_extruded_mesh(xy, cells, z)
    t.set_from_options()
    t.set_constant_tensor_permeability(K.ravel())
    t.set_boundary_pressure_type_function(lambda x, y, z: T.DIRICHLET_BC)
    grad = np.array([1.3e3, -7.0e2, 2.1e3])
    err, scale = _linear_field_fluxes(t, grad, K)
    assert err <= 1e-10 * scale, (err, scale)


def test_hydrostatic_state_has_no_internal_flux():
    """For P = P0 + rho g (z_top - z) with constant rho on an orthogonal box,
    TP + rho G = 0 on every face, so the TS residual with U_t = 0 and
    Dirichlet top at the hydrostatic value vanishes up to rounding."""
    T.options_clear()
    t, U0, _ = W.hydrostatic_box(6, rho=998.0)
    o = Oracle(_host(t))
    R, mag = o.ts_ifunction(U0, np.zeros_like(U0), with_mag=True)
    assert np.all(np.abs(R) <= 1e-12 * np.maximum(mag, 1e-300) + 1e-30)


def test_oracle_threaded_residual_matches_serial():
    """The oracle's threaded residual (vertex colours on threads, used for the
    per-step checks of long runs) equals the serial one to rounding."""
    T.options_clear()
    t, U0, top, src, info = W.infiltration_prisms(300, 6)
    t.setup(host_only=True)
    o = Oracle(t.setup_view())
    rng = np.random.default_rng(3)
    U = U0 + rng.normal(0.0, 3e3, U0.size)
    o.snes_presolve(U + rng.normal(0.0, 50.0, U0.size), 600.0)
    R, M = o.snes_function(U, with_mag=True)
    Rp = o.snes_function_parallel(U, 4)
    assert np.all(np.abs(Rp - R) <= 1e-13 * M)


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's sizes
    and field offsets (a field added on one side only would shift the rest)."""
    import ctypes
    import shutil
    import subprocess
    from pathlib import Path

    import tdycore_gb300 as T

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = Path(__file__).resolve().parent.parent
    fields = {"TDyNewtonStats": T.NewtonStats, "TDyNewtonOptions": T.NewtonOptions}
    lines = []
    for cname, cls in fields.items():
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"tdycore_gb300.h\"\nint main(void) {\n"
                   + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(root / "include"), "-o", str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for cls in fields.values():
        want.append(ctypes.sizeof(cls))
        want += [getattr(cls, f).offset for f, _ in cls._fields_]
    assert got == want


def test_newton_option_defaults():
    """TDyNewtonOptionsDefault (no device needed) sets PETSc's SNES defaults
    and the mixed-precision defaults the documentation states."""
    import ctypes

    o = T.NewtonOptions()
    assert T.lib.TDyNewtonOptionsDefault(ctypes.byref(o)) == 0
    assert (o.rtol, o.atol, o.max_it, o.stol) == (1e-8, 0.0, 50, 1e-8)
    assert (o.linear_fp32, o.linear_rtol, o.linear_max_it) == (1, 1e-6, 400)
    assert (o.precond, o.cluster_threshold) == (T.PRECOND_LINES, 0.05)
    assert (o.schedule, o.fp32_max_it, o.spmv_threads) == (T.SCHEDULE_AUTO, 8, 0)
