"""GB300-native MPFA-O Richards residual/Jacobian (TDycore drop-in path).

Python mirror of the C-ABI in ``include/tdycore_gb300.h``.  The class
:class:`TDy` follows the reference's call sequence (``TDyCreate`` ->
``TDySetMode(RICHARDS)`` -> ``TDySetDiscretization(MPFA_O)`` ->
``TDySetFromOptions`` -> ``TDySetup``) and exposes the SNES and TS forms of
the residual and Jacobian (``TDyMPFAOSNESFunction`` / ``TDyMPFAOSNESJacobian``
in src/fv/mpfao/tdympfao_snes.c, ``TDyMPFAOIFunction`` / ``TDyMPFAOIJacobian``
in src/fv/mpfao/tdympfao_ts.c).

All evaluation runs in the CUDA library; there is no CPU fallback.  Importing
this package fails if the shared library has not been built.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_char_p, c_double, c_int, c_longlong, c_void_p
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libtdycore_gb300.so"
if not _LIB_PATH.exists():
    raise ImportError(
        f"{_LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
        "(nvcc, sm_103a)"
    )
lib = ctypes.CDLL(str(_LIB_PATH))

# enums (include/tdycore.h)
RICHARDS, TH, SALINITY = 0, 1, 2
MPFA_O, MPFA_O_DAE, MPFA_O_TRANSIENTVAR, BDM, WY, FV_TPF = range(6)
MPFAO_GMATRIX_DEFAULT, MPFAO_GMATRIX_TPF = 0, 1
DIRICHLET_BC, NEUMANN_BC, SEEPAGE_BC = 0, 1, 2
WATER_DENSITY_CONSTANT, WATER_DENSITY_EXPONENTIAL, WATER_DENSITY_BATZLE_AND_WANG = 0, 1, 2
WATER_VISCOSITY_CONSTANT, WATER_VISCOSITY_BATZLE_AND_WANG = 0, 1

TDY_ERR_GPU = 97

_dp = POINTER(c_double)
_ip = POINTER(c_int)

ScalarSpatialFunction = ctypes.CFUNCTYPE(None, c_int, _dp, _dp)
IntegerSpatialFunction = ctypes.CFUNCTYPE(None, c_int, _dp, _ip)


class TDyMPFAOSetupView(ctypes.Structure):
    """ctypes image of ``struct TDyMPFAOSetupView`` (include/tdycore_gb300_setup.h)."""

    _fields_ = [
        ("ncells", c_int), ("nfaces", c_int), ("nbnd", c_int), ("nverts", c_int),
        ("nrows_total", c_int), ("ncols_total", c_int), ("ntrans_total", c_longlong),
        ("bc_type", c_int), ("gmatrix_method", c_int), ("rho_type", c_int), ("mu_type", c_int),
        ("gravity", c_double), ("Pref", c_double),
        ("volume", _dp), ("centroid", _dp), ("porosity", _dp), ("Sr", _dp), ("K0", _dp),
        ("sat_type", _ip), ("sat_param", _dp), ("relperm_type", _ip), ("relperm_param", _dp),
        ("source_sink", _dp),
        ("face_up", _ip), ("face_dn", _ip), ("gravdis", _dp), ("face_centroid", _dp),
        ("face_area", _dp), ("face_normal", _dp), ("face_nverts", _ip),
        ("bnd_face", _ip), ("bnd_type", _ip), ("bnd_has_value", _ip), ("bnd_value", _dp),
        ("rho_bnd", _dp), ("vis_bnd", _dp),
        ("v_row_off", _ip), ("v_col_off", _ip), ("v_nint", _ip), ("v_trans_off", POINTER(c_longlong)),
        ("row_face", _ip), ("col_ext", _ip), ("trans", _dp),
        ("rowptr", _ip), ("colidx", _ip), ("nnz", c_int),
    ]


class NewtonOptions(ctypes.Structure):
    _fields_ = [("rtol", c_double), ("atol", c_double), ("max_it", c_int), ("linear_fp32", c_int),
                ("linear_rtol", c_double), ("linear_max_it", c_int), ("stol", c_double), ("precond", c_int),
                ("cluster_threshold", c_double), ("schedule", c_int), ("fp32_max_it", c_int),
                ("spmv_threads", c_int)]


PRECOND_LINES, PRECOND_CLUSTERS = 0, 1
SCHEDULE_AUTO, SCHEDULE_TILE, SCHEDULE_BLOCK = 0, 1, 2


class NewtonStats(ctypes.Structure):
    _fields_ = [("newton_iterations", c_int), ("linear_iterations", c_longlong), ("converged", c_int),
                ("ninstances", c_int), ("max_rel_residual", c_double), ("step_converged", c_int),
                ("precond_used", c_int), ("clusters", c_int), ("cluster_cells", c_int),
                ("cluster_cells_diagonal", c_int), ("block_instances", c_int), ("block_max_cells", c_longlong),
                ("fp64_fallback", c_int), ("eval_schedule", c_int), ("eval_s", c_double), ("precond_s", c_double),
                ("krylov_s", c_double), ("fp64_inner_redo", c_int)]


def _sig(name, *args):
    f = getattr(lib, name)
    f.argtypes = list(args)
    f.restype = c_int
    return f


lib.TDyGetErrorMessage.restype = c_char_p
lib.TDyGetErrorMessage.argtypes = []
_sig("TDyInit", c_int, c_void_p)
_sig("TDyOptionsInsertString", c_char_p)
_sig("TDyOptionsClear")
_sig("TDyOptionsGetReal", c_char_p, _dp, _ip)
_sig("TDyOptionsGetInt", c_char_p, _ip, _ip)
_sig("TDyOptionsGetString", c_char_p, c_char_p, c_int, _ip)
_sig("TDyOptionsHasName", c_char_p, _ip)
_sig("TDyOutputRegression", c_void_p, _dp)
_sig("TDyNewtonOptionsDefault", POINTER(NewtonOptions))
_sig("TDyGetNumInstances", c_void_p, _ip)
_sig("TDySetActiveInstances", c_void_p, c_int, _ip)
_sig("TDyGetInstanceStatus", c_void_p, c_int, _ip)
INSTANCE_NOT_CONVERGED, INSTANCE_CONVERGED, INSTANCE_STEP_TEST, INSTANCE_INACTIVE = 0, 1, 2, 3
_sig("TDyBackwardEulerStepDevice", c_void_p, c_double, c_void_p, POINTER(NewtonOptions), POINTER(NewtonStats), _ip,
     _dp, c_void_p)
_sig("TDyCreate", c_void_p, POINTER(c_void_p))
_sig("TDyDestroy", POINTER(c_void_p))
_sig("TDySetMode", c_void_p, c_int)
_sig("TDySetDiscretization", c_void_p, c_int)
_sig("TDySetDiscretizationMethod", c_void_p, c_int)
_sig("TDySetFromOptions", c_void_p)
_sig("TDySetup", c_void_p)
_sig("TDySetupHost", c_void_p)
_sig("TDySetBoxMesh", c_void_p, c_int, c_int, c_int, _dp, _dp)
_sig("TDySetExtrudedMesh", c_void_p, c_int, _dp, c_int, c_int, _ip, c_int, _dp)
_sig("TDySetExtrudedMeshes", c_void_p, c_int, _ip, _dp, _ip, c_int, _ip, _ip, _dp)
_sig("TDySetWaterDensityType", c_void_p, c_int)
_sig("TDySetWaterViscosityType", c_void_p, c_int)
_sig("TDySetConstantPorosity", c_void_p, c_double)
_sig("TDySetPorosityFunction", c_void_p, ScalarSpatialFunction)
_sig("TDySetConstantIsotropicPermeability", c_void_p, c_double)
_sig("TDySetConstantDiagonalPermeability", c_void_p, _dp)
_sig("TDySetConstantTensorPermeability", c_void_p, _dp)
_sig("TDySetConstantResidualSaturation", c_void_p, c_double)
_sig("TDySetPorosityValuesLocal", c_void_p, c_int, _ip, _dp)
_sig("TDySetPermeabilityValuesLocal", c_void_p, c_int, _ip, _dp)
_sig("TDySetResidualSaturationValuesLocal", c_void_p, c_int, _ip, _dp)
_sig("TDySetCharacteristicCurveVanGenuchtenValuesLocal", c_void_p, c_int, _ip, _dp, _dp)
_sig("TDySetCharacteristicCurveMualemValuesLocal", c_void_p, c_int, _ip, _dp)
_sig("TDySetCharacteristicCurveGardnerValuesLocal", c_void_p, c_int, _ip, _dp, _dp, _dp)
_sig("TDySetCharacteristicCurveIrmayValuesLocal", c_void_p, c_int, _ip, _dp)
_sig("TDySetSourceSinkValuesLocal", c_void_p, c_int, _ip, _dp)
_sig("TDySetBoundaryPressureFunction", c_void_p, ScalarSpatialFunction)
_sig("TDySetBoundaryPressureTypeFunction", c_void_p, IntegerSpatialFunction)
_sig("TDyMPFAOSetGmatrixMethod", c_void_p, c_int)
_sig("TDyMPFAOSetBoundaryConditionType", c_void_p, c_int)
_sig("TDyGetNumCells", c_void_p, _ip)
_sig("TDyGetNumBoundaryFaces", c_void_p, _ip)
_sig("TDyGetCellCentroids", c_void_p, _dp)
_sig("TDyGetCellVolumes", c_void_p, _dp)
_sig("TDyGetJacobianPattern", c_void_p, _ip, _ip, POINTER(_ip), POINTER(_ip))
_sig("TDyCreateVectors", c_void_p)
_sig("TDyCreateJacobian", c_void_p)
_sig("TDySetDtimeForSNESSolver", c_void_p, c_double)
_sig("TDySetPreviousSolutionForSNESSolver", c_void_p, _dp)
_sig("TDyPreSolveSNESSolver", c_void_p)
_sig("TDyPostSolve", c_void_p, _dp)
_sig("TDyMPFAOSNESFunction", c_void_p, _dp, _dp)
_sig("TDyMPFAOSNESJacobian", c_void_p, _dp, _dp)
_sig("TDyMPFAOSNESFunctionJacobian", c_void_p, _dp, _dp, _dp)
_sig("TDyMPFAOIFunction", c_void_p, c_double, _dp, _dp, _dp)
_sig("TDyMPFAOIJacobian", c_void_p, c_double, _dp, _dp, c_double, _dp)
_sig("TDyMPFAOIFunctionIJacobian", c_void_p, c_double, _dp, _dp, c_double, _dp, _dp)
_sig("TDyMPFAOTransientVariable", c_void_p, _dp, _dp)
_sig("TDyMPFAOTransientVariableDerivative", c_void_p, _dp, _dp)
_sig("TDyMPFAOIFunctionTransientVariable", c_void_p, c_double, _dp, _dp, _dp)
_sig("TDyMPFAOIJacobianTransientVariable", c_void_p, c_double, _dp, c_double, _dp)
_sig("TDyMPFAOIFunctionDAE", c_void_p, c_double, _dp, _dp, _dp)
_sig("TDyMPFAOSNESFunctionJacobianDevice", c_void_p, c_void_p, c_void_p, c_void_p, c_void_p)
_sig("TDyMPFAOIFunctionIJacobianDevice", c_void_p, c_double, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
     c_void_p)
_sig("TDyPreSolveSNESSolverDevice", c_void_p, c_void_p, c_void_p)
_sig("TDyMPFAOSNESFunctionJacobianDeviceNoAlloc", c_void_p, c_void_p, c_void_p, c_void_p, c_void_p)
_sig("TDyMPFAOSNESFunctionJacobianDeviceInstances", c_void_p, c_void_p, c_void_p, c_void_p, c_int, _ip, c_void_p)
_sig("TDyGetLaunchesPerEvaluation", c_void_p, _ip)
_sig("TDySynchronize", c_void_p)
_sig("TDyUpdateState", c_void_p, _dp, c_int)
_sig("TDyGetLiquidSaturation", c_void_p, _dp)
_sig("TDyGetLiquidMass", c_void_p, _dp)
_sig("TDyMPFAOGetSetupView", c_void_p, POINTER(TDyMPFAOSetupView))
_sig("TDySetTimersEnabled", c_void_p, c_int)
_sig("TDyGetTimers", c_void_p, _ip, POINTER(c_char_p), _dp, POINTER(c_longlong))
_sig("TDyDeviceFP64Throughput", _dp)


def device_fp64_tflops() -> float:
    """Measured FP64 FMA throughput of the current CUDA device."""
    x = c_double()
    check(lib.TDyDeviceFP64Throughput(byref(x)), "TDyDeviceFP64Throughput")
    return x.value


class TDyError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib.TDyGetErrorMessage().decode(errors="replace")
        super().__init__(f"{where} failed with TDyErrorCode {code}: {msg}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != 0:
        raise TDyError(code, where)


def _as_dp(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _f64(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def options_insert(options: str) -> None:
    check(lib.TDyOptionsInsertString(options.encode()), "TDyOptionsInsertString")


def options_clear() -> None:
    check(lib.TDyOptionsClear(), "TDyOptionsClear")


def options_get_real(name: str, default=None):
    """PetscOptionsGetReal analogue: the option's value, or ``default``."""
    v, f = c_double(), c_int()
    check(lib.TDyOptionsGetReal(name.encode(), byref(v), byref(f)), "TDyOptionsGetReal")
    return v.value if f.value else default


def options_get_int(name: str, default=None):
    v, f = c_int(), c_int()
    check(lib.TDyOptionsGetInt(name.encode(), byref(v), byref(f)), "TDyOptionsGetInt")
    return v.value if f.value else default


def options_get_string(name: str, default=None):
    buf, f = ctypes.create_string_buffer(4096), c_int()
    check(lib.TDyOptionsGetString(name.encode(), buf, 4096, byref(f)), "TDyOptionsGetString")
    return buf.value.decode() if f.value else default


def options_has_name(name: str) -> bool:
    f = c_int()
    check(lib.TDyOptionsHasName(name.encode(), byref(f)), "TDyOptionsHasName")
    return bool(f.value)


def _eval_points(f, n, x, out, dtype):
    """Evaluates f(x, y, z) at n points (x: 3n doubles) into out: once on
    numpy arrays when f accepts them, else point by point."""
    pts = np.ctypeslib.as_array(x, shape=(3 * n,)).reshape(n, 3)
    res = np.ctypeslib.as_array(out, shape=(n,))
    try:
        v = np.asarray(f(pts[:, 0], pts[:, 1], pts[:, 2]))
        if v.shape in ((), (n,)):
            res[:] = np.broadcast_to(v, (n,)).astype(dtype)
            return
    except (TypeError, ValueError):
        pass
    for i in range(n):
        res[i] = dtype(f(*pts[i]))


class TDy:
    """One MPFA-O Richards instance; owns its device buffers."""

    def __init__(self):
        self._h = c_void_p()
        check(lib.TDyCreate(None, byref(self._h)), "TDyCreate")
        self.discretization = MPFA_O
        self._keep = []  # ctypes callbacks must outlive the handle
        self.ncells = 0
        self.nnz = 0

    # lifecycle -------------------------------------------------------------
    def set_mode(self, mode=RICHARDS):
        check(lib.TDySetMode(self._h, mode), "TDySetMode")
        return self

    def set_discretization(self, disc=MPFA_O):
        check(lib.TDySetDiscretization(self._h, disc), "TDySetDiscretization")
        self.discretization = disc
        return self

    def set_from_options(self):
        check(lib.TDySetFromOptions(self._h), "TDySetFromOptions")
        return self

    def setup(self, host_only: bool = False):
        if host_only:
            check(lib.TDySetupHost(self._h), "TDySetupHost")
        else:
            check(lib.TDySetup(self._h), "TDySetup")
        n = c_int()
        check(lib.TDyGetNumCells(self._h, byref(n)), "TDyGetNumCells")
        self.ncells = n.value
        nr, nnz = c_int(), c_int()
        rp, ci = _ip(), _ip()
        check(lib.TDyGetJacobianPattern(self._h, byref(nr), byref(nnz), byref(rp), byref(ci)), "TDyGetJacobianPattern")
        self.nnz = nnz.value
        self.rowptr = np.ctypeslib.as_array(rp, shape=(nr.value + 1,)).copy()
        self.colidx = np.ctypeslib.as_array(ci, shape=(nnz.value,)).copy()
        return self

    def destroy(self):
        if self._h:
            lib.TDyDestroy(byref(self._h))
            self._h = c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # mesh ------------------------------------------------------------------
    def set_box_mesh(self, nx, ny, nz, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
        lo, hi = _f64(lower, 3), _f64(upper, 3)
        check(lib.TDySetBoxMesh(self._h, nx, ny, nz, _as_dp(lo), _as_dp(hi)), "TDySetBoxMesh")
        return self

    def set_extruded_mesh(self, xy, cells2d, z):
        xy = _f64(xy).reshape(-1, 2)
        cells2d = _i32(cells2d)
        nvpc = cells2d.shape[1]
        z = _f64(z).reshape(-1, xy.shape[0])
        check(lib.TDySetExtrudedMesh(self._h, xy.shape[0], _as_dp(xy), cells2d.shape[0], nvpc,
                                     cells2d.ctypes.data_as(_ip), z.shape[0] - 1, _as_dp(z)), "TDySetExtrudedMesh")
        return self

    def set_extruded_meshes(self, blocks):
        """A batch of independent extruded meshes: ``blocks`` is a list of
        (xy, cells2d, z) as for set_extruded_mesh (same polygon size)."""
        nvpc = {np.asarray(c).shape[1] for _, c, _ in blocks}
        if len(nvpc) != 1:
            raise ValueError("all blocks must use the same polygon size")
        nvpc = nvpc.pop()
        xys = [_f64(xy).reshape(-1, 2) for xy, _, _ in blocks]
        nv2 = _i32([a.shape[0] for a in xys])
        nc2 = _i32([np.asarray(c).shape[0] for _, c, _ in blocks])
        zs = [_f64(z).reshape(-1, a.shape[0]) for (_, _, z), a in zip(blocks, xys)]
        nl = _i32([z.shape[0] - 1 for z in zs])
        xy = _f64(np.concatenate([a.ravel() for a in xys]))
        c2 = _i32(np.concatenate([np.asarray(c, dtype=np.int32).ravel() for _, c, _ in blocks]))
        z = _f64(np.concatenate([a.ravel() for a in zs]))
        check(lib.TDySetExtrudedMeshes(self._h, len(blocks), nv2.ctypes.data_as(_ip), _as_dp(xy),
                                       nc2.ctypes.data_as(_ip), nvpc, c2.ctypes.data_as(_ip), nl.ctypes.data_as(_ip),
                                       _as_dp(z)), "TDySetExtrudedMeshes")
        self.block_cells = np.concatenate([[0], np.cumsum(nc2.astype(np.int64) * nl)])
        return self

    # materials --------------------------------------------------------------
    def set_water_density_type(self, t):
        check(lib.TDySetWaterDensityType(self._h, t), "TDySetWaterDensityType")
        return self

    def set_water_viscosity_type(self, t):
        check(lib.TDySetWaterViscosityType(self._h, t), "TDySetWaterViscosityType")
        return self

    def set_constant_porosity(self, v):
        check(lib.TDySetConstantPorosity(self._h, v), "TDySetConstantPorosity")
        return self

    def set_porosity_function(self, f):
        cb = ScalarSpatialFunction(f)
        self._keep.append(cb)
        check(lib.TDySetPorosityFunction(self._h, cb), "TDySetPorosityFunction")
        return self

    def set_constant_isotropic_permeability(self, k):
        check(lib.TDySetConstantIsotropicPermeability(self._h, k), "TDySetConstantIsotropicPermeability")
        return self

    def set_constant_diagonal_permeability(self, k3):
        k = _f64(k3, 3)
        check(lib.TDySetConstantDiagonalPermeability(self._h, _as_dp(k)), "TDySetConstantDiagonalPermeability")
        return self

    def set_constant_tensor_permeability(self, k9):
        k = _f64(k9, 9)
        check(lib.TDySetConstantTensorPermeability(self._h, _as_dp(k)), "TDySetConstantTensorPermeability")
        return self

    def set_constant_residual_saturation(self, v):
        check(lib.TDySetConstantResidualSaturation(self._h, v), "TDySetConstantResidualSaturation")
        return self

    def _cells(self, cells, n):
        if cells is None:
            return None, None
        c = _i32(cells)
        if c.size != n:
            raise ValueError("cells and values differ in length")
        return c, c.ctypes.data_as(_ip)

    def set_porosity_values(self, vals, cells=None):
        v = _f64(vals)
        c, cp = self._cells(cells, v.size)
        check(lib.TDySetPorosityValuesLocal(self._h, v.size, cp, _as_dp(v)), "TDySetPorosityValuesLocal")
        return self

    def set_permeability_values(self, k9, cells=None):
        k = _f64(k9).reshape(-1, 9)
        c, cp = self._cells(cells, k.shape[0])
        check(lib.TDySetPermeabilityValuesLocal(self._h, k.shape[0], cp, _as_dp(k)), "TDySetPermeabilityValuesLocal")
        return self

    def set_residual_saturation_values(self, vals, cells=None):
        v = _f64(vals)
        c, cp = self._cells(cells, v.size)
        check(lib.TDySetResidualSaturationValuesLocal(self._h, v.size, cp, _as_dp(v)),
              "TDySetResidualSaturationValuesLocal")
        return self

    def set_vangenuchten_values(self, m, alpha, cells=None):
        m, a = _f64(m), _f64(alpha)
        c, cp = self._cells(cells, m.size)
        check(lib.TDySetCharacteristicCurveVanGenuchtenValuesLocal(self._h, m.size, cp, _as_dp(m), _as_dp(a)),
              "TDySetCharacteristicCurveVanGenuchtenValuesLocal")
        return self

    def set_mualem_values(self, m, cells=None):
        m = _f64(m)
        c, cp = self._cells(cells, m.size)
        check(lib.TDySetCharacteristicCurveMualemValuesLocal(self._h, m.size, cp, _as_dp(m)),
              "TDySetCharacteristicCurveMualemValuesLocal")
        return self

    def set_gardner_values(self, n, m, alpha, cells=None):
        n, m, a = _f64(n), _f64(m), _f64(alpha)
        c, cp = self._cells(cells, n.size)
        check(lib.TDySetCharacteristicCurveGardnerValuesLocal(self._h, n.size, cp, _as_dp(n), _as_dp(m), _as_dp(a)),
              "TDySetCharacteristicCurveGardnerValuesLocal")
        return self

    def set_irmay_values(self, m, cells=None):
        m = _f64(m)
        c, cp = self._cells(cells, m.size)
        check(lib.TDySetCharacteristicCurveIrmayValuesLocal(self._h, m.size, cp, _as_dp(m)),
              "TDySetCharacteristicCurveIrmayValuesLocal")
        return self

    def set_source_sink_values(self, q, cells=None):
        q = _f64(q)
        c, cp = self._cells(cells, q.size)
        check(lib.TDySetSourceSinkValuesLocal(self._h, q.size, cp, _as_dp(q)), "TDySetSourceSinkValuesLocal")
        return self

    # boundary conditions ------------------------------------------------------
    def set_boundary_pressure_function(self, f):
        """f(x, y, z) -> pressure, evaluated once per boundary face centroid."""

        def wrapped(n, x, out):
            _eval_points(f, n, x, out, np.float64)

        cb = ScalarSpatialFunction(wrapped)
        self._keep.append(cb)
        check(lib.TDySetBoundaryPressureFunction(self._h, cb), "TDySetBoundaryPressureFunction")
        return self

    def set_boundary_pressure_type_function(self, f):
        """f(x, y, z) -> DIRICHLET_BC | NEUMANN_BC | SEEPAGE_BC per boundary face."""

        def wrapped(n, x, out):
            _eval_points(f, n, x, out, np.int32)

        cb = IntegerSpatialFunction(wrapped)
        self._keep.append(cb)
        check(lib.TDySetBoundaryPressureTypeFunction(self._h, cb), "TDySetBoundaryPressureTypeFunction")
        return self

    def set_gmatrix_method(self, m):
        check(lib.TDyMPFAOSetGmatrixMethod(self._h, m), "TDyMPFAOSetGmatrixMethod")
        return self

    def set_boundary_condition_type(self, t):
        check(lib.TDyMPFAOSetBoundaryConditionType(self._h, t), "TDyMPFAOSetBoundaryConditionType")
        return self

    # queries ----------------------------------------------------------------
    def cell_centroids(self):
        x = np.empty((self.ncells, 3))
        check(lib.TDyGetCellCentroids(self._h, _as_dp(x)), "TDyGetCellCentroids")
        return x

    def cell_volumes(self):
        v = np.empty(self.ncells)
        check(lib.TDyGetCellVolumes(self._h, _as_dp(v)), "TDyGetCellVolumes")
        return v

    def setup_view(self) -> dict:
        """Copies of the setup arrays (layout: include/tdycore_gb300_setup.h)."""
        v = TDyMPFAOSetupView()
        check(lib.TDyMPFAOGetSetupView(self._h, byref(v)), "TDyMPFAOGetSetupView")
        nc, nf, nb, nv = v.ncells, v.nfaces, v.nbnd, v.nverts

        def arr(p, n):
            return np.ctypeslib.as_array(p, shape=(n,)).copy() if n > 0 else np.zeros(0)

        d = {k: getattr(v, k) for k in ("ncells", "nfaces", "nbnd", "nverts", "nrows_total", "ncols_total",
                                        "ntrans_total", "bc_type", "gmatrix_method", "rho_type", "mu_type",
                                        "gravity", "Pref", "nnz")}
        for k, n in (("volume", nc), ("centroid", 3 * nc), ("porosity", nc), ("Sr", nc), ("K0", 9 * nc),
                     ("sat_type", nc), ("sat_param", 3 * nc), ("relperm_type", nc), ("relperm_param", 9 * nc),
                     ("source_sink", nc), ("face_up", nf), ("face_dn", nf), ("gravdis", nf),
                     ("face_centroid", 3 * nf), ("face_area", nf), ("face_normal", 3 * nf), ("face_nverts", nf),
                     ("bnd_face", nb), ("bnd_type", nb), ("bnd_has_value", nb), ("bnd_value", nb),
                     ("rho_bnd", nb), ("vis_bnd", nb), ("v_row_off", nv + 1), ("v_col_off", nv + 1),
                     ("v_nint", nv), ("v_trans_off", nv + 1), ("row_face", v.nrows_total),
                     ("col_ext", v.ncols_total), ("trans", v.ntrans_total), ("rowptr", nc + 1),
                     ("colidx", v.nnz)):
            d[k] = arr(getattr(v, k), n)
        return d

    # SNES form ----------------------------------------------------------------
    def set_dtime(self, dt):
        check(lib.TDySetDtimeForSNESSolver(self._h, dt), "TDySetDtimeForSNESSolver")

    def presolve(self, U_prev):
        """TDySetPreviousSolutionForSNESSolver + TDyPreSolveSNESSolver."""
        self.set_previous_solution(U_prev)
        self.presolve_current()

    def set_previous_solution(self, U_prev):
        u = _f64(U_prev, self.ncells)
        check(lib.TDySetPreviousSolutionForSNESSolver(self._h, _as_dp(u)), "TDySetPreviousSolutionForSNESSolver")

    def presolve_current(self):
        """TDyPreSolveSNESSolver: accumulation at the stored previous solution."""
        check(lib.TDyPreSolveSNESSolver(self._h), "TDyPreSolveSNESSolver")

    def post_solve(self, U):
        """TDyPostSolve: U becomes the previous solution."""
        u = _f64(U, self.ncells)
        check(lib.TDyPostSolve(self._h, _as_dp(u)), "TDyPostSolve")

    def snes_function(self, U):
        u = _f64(U, self.ncells)
        R = np.empty(self.ncells)
        check(lib.TDyMPFAOSNESFunction(self._h, _as_dp(u), _as_dp(R)), "TDyMPFAOSNESFunction")
        return R

    def snes_jacobian(self, U):
        u = _f64(U, self.ncells)
        J = np.empty(self.nnz)
        check(lib.TDyMPFAOSNESJacobian(self._h, _as_dp(u), _as_dp(J)), "TDyMPFAOSNESJacobian")
        return J

    def snes_function_jacobian(self, U, R=None, J=None):
        """Fused residual + Jacobian; R and J may be caller-owned (e.g. pinned) float64 arrays."""
        u = _f64(U, self.ncells)
        R = np.empty(self.ncells) if R is None else R
        J = np.empty(self.nnz) if J is None else J
        if R.dtype != np.float64 or J.dtype != np.float64 or not (R.flags.c_contiguous and J.flags.c_contiguous):
            raise ValueError("R and J must be contiguous float64 arrays")
        if R.size != self.ncells or J.size != self.nnz:
            raise ValueError("R or J has the wrong size")
        check(lib.TDyMPFAOSNESFunctionJacobian(self._h, _as_dp(u), _as_dp(R), _as_dp(J)),
              "TDyMPFAOSNESFunctionJacobian")
        return R, J

    # TS form ----------------------------------------------------------------
    def ifunction(self, t, U, Ut):
        u, ut = _f64(U, self.ncells), _f64(Ut, self.ncells)
        R = np.empty(self.ncells)
        check(lib.TDyMPFAOIFunction(self._h, t, _as_dp(u), _as_dp(ut), _as_dp(R)), "TDyMPFAOIFunction")
        return R

    def ijacobian(self, t, U, Ut, shift):
        u, ut = _f64(U, self.ncells), _f64(Ut, self.ncells)
        J = np.empty(self.nnz)
        check(lib.TDyMPFAOIJacobian(self._h, t, _as_dp(u), _as_dp(ut), shift, _as_dp(J)), "TDyMPFAOIJacobian")
        return J

    def ifunction_ijacobian(self, t, U, Ut, shift):
        u, ut = _f64(U, self.ncells), _f64(Ut, self.ncells)
        R = np.empty(self.ncells)
        J = np.empty(self.nnz)
        check(lib.TDyMPFAOIFunctionIJacobian(self._h, t, _as_dp(u), _as_dp(ut), shift, _as_dp(R), _as_dp(J)),
              "TDyMPFAOIFunctionIJacobian")
        return R, J

    # transient-variable and DAE forms ----------------------------------------
    def transient_variable(self, U, with_derivative=False):
        u = _f64(U, self.ncells)
        C = np.empty(self.ncells)
        check(lib.TDyMPFAOTransientVariable(self._h, _as_dp(u), _as_dp(C)), "TDyMPFAOTransientVariable")
        if not with_derivative:
            return C
        dC = np.empty(self.ncells)
        check(lib.TDyMPFAOTransientVariableDerivative(self._h, _as_dp(u), _as_dp(dC)),
              "TDyMPFAOTransientVariableDerivative")
        return C, dC

    def tv_ifunction(self, t, U, M_t):
        u, m = _f64(U, self.ncells), _f64(M_t, self.ncells)
        R = np.empty(self.ncells)
        check(lib.TDyMPFAOIFunctionTransientVariable(self._h, t, _as_dp(u), _as_dp(m), _as_dp(R)),
              "TDyMPFAOIFunctionTransientVariable")
        return R

    def tv_ijacobian(self, t, U, shift):
        u = _f64(U, self.ncells)
        J = np.empty(self.nnz)
        check(lib.TDyMPFAOIJacobianTransientVariable(self._h, t, _as_dp(u), shift, _as_dp(J)),
              "TDyMPFAOIJacobianTransientVariable")
        return J

    def dae_ifunction(self, t, U, U_t):
        u, ut = _f64(U, 2 * self.ncells), _f64(U_t, 2 * self.ncells)
        R = np.empty(2 * self.ncells)
        check(lib.TDyMPFAOIFunctionDAE(self._h, t, _as_dp(u), _as_dp(ut), _as_dp(R)), "TDyMPFAOIFunctionDAE")
        return R

    # device Newton -------------------------------------------------------------
    def num_instances(self) -> int:
        n = c_int()
        check(lib.TDyGetNumInstances(self._h, byref(n)), "TDyGetNumInstances")
        return n.value

    def set_active_instances(self, active=None):
        """Instances the next device Newton steps advance (None: all)."""
        if active is None:
            check(lib.TDySetActiveInstances(self._h, 0, None), "TDySetActiveInstances")
            return
        a = _i32(active)
        check(lib.TDySetActiveInstances(self._h, a.size, a.ctypes.data_as(_ip)), "TDySetActiveInstances")

    def instance_status(self):
        """Per-instance outcome of the last device Newton step (INSTANCE_*)."""
        n = self.num_instances()
        st = np.zeros(n, dtype=np.int32)
        check(lib.TDyGetInstanceStatus(self._h, n, st.ctypes.data_as(_ip)), "TDyGetInstanceStatus")
        return st

    def backward_euler_step_device(self, dU, dt, rtol=1e-8, atol=0.0, max_it=50, fp32=True, linear_rtol=1e-6,
                                   linear_max_it=400, stol=1e-8, stream=None, precond="lines",
                                   cluster_threshold=0.05, schedule="auto", fp32_max_it=8, spmv_threads=0):
        """One backward-Euler step of every instance with the device Newton
        solver; dU (device float64 tensor, ncells) holds U_n and receives
        U_{n+1}.  precond: "lines" or "clusters" (TDY_PRECOND_*); schedule:
        "auto", "tile" or "block" (TDY_SCHEDULE_*, the same bits); with
        fp32, inner solves switch to FP64 after fp32_max_it Newton iterations
        (negative: never); spmv_threads: threads per row of the inner solve's
        sparse products (0: timed; 1, 2, 4, 8: the same bits).  Returns
        (stats dict, per-instance Newton iterations, per-instance final
        ||F||/||F_0||)."""
        o = NewtonOptions()
        check(lib.TDyNewtonOptionsDefault(byref(o)), "TDyNewtonOptionsDefault")
        o.rtol, o.atol, o.max_it, o.linear_fp32 = rtol, atol, max_it, int(bool(fp32))
        o.linear_rtol, o.linear_max_it, o.stol = linear_rtol, linear_max_it, stol
        o.precond = {"lines": PRECOND_LINES, "clusters": PRECOND_CLUSTERS}[precond]
        o.cluster_threshold = cluster_threshold
        o.schedule = {"auto": SCHEDULE_AUTO, "tile": SCHEDULE_TILE, "block": SCHEDULE_BLOCK}[schedule]
        o.fp32_max_it = fp32_max_it
        o.spmv_threads = spmv_threads
        st = NewtonStats()
        ni = self.num_instances()
        its = np.zeros(ni, dtype=np.int32)
        rel = np.zeros(ni)
        check(lib.TDyBackwardEulerStepDevice(self._h, dt, self._ptr(dU), byref(o), byref(st),
                                             its.ctypes.data_as(_ip), _as_dp(rel), self._ptr(stream)),
              "TDyBackwardEulerStepDevice")
        stats = {k: getattr(st, k) for k, _ in NewtonStats._fields_}
        return stats, its, rel

    # device-pointer forms (torch tensors or raw pointers) -------------------
    @staticmethod
    def _ptr(x):
        if x is None:
            return None
        if isinstance(x, int):
            return c_void_p(x)
        return c_void_p(x.data_ptr())

    def snes_function_jacobian_device(self, dU, dR, dJ, stream=None):
        check(lib.TDyMPFAOSNESFunctionJacobianDevice(self._h, self._ptr(dU), self._ptr(dR), self._ptr(dJ),
                                                     self._ptr(stream) if stream is not None else None),
              "TDyMPFAOSNESFunctionJacobianDevice")

    def snes_function_jacobian_device_instances(self, dU, dR, dJ, instances, stream=None):
        """SNES R and J of the listed instances of a batched handle only (one
        CTA per instance); the other rows of dR and dJ are left as they are."""
        lst = _i32(instances)
        check(lib.TDyMPFAOSNESFunctionJacobianDeviceInstances(self._h, self._ptr(dU), self._ptr(dR), self._ptr(dJ),
                                                              lst.size, lst.ctypes.data_as(_ip),
                                                              self._ptr(stream) if stream is not None else None),
              "TDyMPFAOSNESFunctionJacobianDeviceInstances")

    def ifunction_ijacobian_device(self, t, dU, dUt, shift, dR, dJ, stream=None):
        check(lib.TDyMPFAOIFunctionIJacobianDevice(self._h, t, self._ptr(dU), self._ptr(dUt), shift, self._ptr(dR),
                                                   self._ptr(dJ),
                                                   self._ptr(stream) if stream is not None else None),
              "TDyMPFAOIFunctionIJacobianDevice")

    def presolve_device(self, dU_prev, stream=None):
        check(lib.TDyPreSolveSNESSolverDevice(self._h, self._ptr(dU_prev),
                                              self._ptr(stream) if stream is not None else None),
              "TDyPreSolveSNESSolverDevice")

    def launches_per_evaluation(self) -> int:
        n = c_int()
        check(lib.TDyGetLaunchesPerEvaluation(self._h, byref(n)), "TDyGetLaunchesPerEvaluation")
        return n.value

    def synchronize(self):
        check(lib.TDySynchronize(self._h), "TDySynchronize")

    # timers -----------------------------------------------------------------
    def set_timers(self, on: bool):
        check(lib.TDySetTimersEnabled(self._h, 1 if on else 0), "TDySetTimersEnabled")

    def timers(self) -> dict:
        n = c_int(8)
        names = (c_char_p * 8)()
        ms = (c_double * 8)()
        calls = (c_longlong * 8)()
        check(lib.TDyGetTimers(self._h, byref(n), names, ms, calls), "TDyGetTimers")
        return {names[i].decode(): (ms[i], calls[i]) for i in range(n.value)}

    def output_regression(self, U):
        """TDyOutputRegression: writes <filename>.regression when
        -tdy_regression_test is set."""
        u = _f64(U, self.ncells)
        check(lib.TDyOutputRegression(self._h, _as_dp(u)), "TDyOutputRegression")

    # diagnostics ------------------------------------------------------------
    def update_state(self, U):
        u = _f64(U, self.ncells)
        check(lib.TDyUpdateState(self._h, _as_dp(u), self.ncells), "TDyUpdateState")

    def liquid_saturation(self):
        s = np.empty(self.ncells)
        check(lib.TDyGetLiquidSaturation(self._h, _as_dp(s)), "TDyGetLiquidSaturation")
        return s

    def liquid_mass(self):
        s = np.empty(self.ncells)
        check(lib.TDyGetLiquidMass(self._h, _as_dp(s)), "TDyGetLiquidMass")
        return s


def create_richards_mpfao() -> TDy:
    """TDyCreate + TDySetMode(RICHARDS) + TDySetDiscretization(MPFA_O)."""
    t = TDy()
    t.set_mode(RICHARDS)
    t.set_discretization(MPFA_O)
    return t
