"""TEST INFRASTRUCTURE ONLY: Python bridge to the C oracle (mpfao_oracle.c).

Imported by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg
of ``bench.py``, never by the product package.  ``Oracle`` takes the setup
arrays exported by ``TDy.setup_view()`` and evaluates the reference's
MPFA-O residual and Jacobian on the CPU.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_longlong, c_void_p
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB = _HERE / "_build" / "libmpfao_oracle.so"

_dp = POINTER(c_double)
_ip = POINTER(c_int)


class OracleInput(ctypes.Structure):
    _fields_ = [
        ("ncells", c_int), ("nfaces", c_int), ("nbnd", c_int), ("nverts", c_int),
        ("bc_type", c_int), ("rho_type", c_int), ("mu_type", c_int),
        ("Pref", c_double),
        ("volume", _dp), ("porosity", _dp), ("Sr", _dp),
        ("sat_type", _ip), ("sat_param", _dp), ("relperm_type", _ip), ("relperm_param", _dp),
        ("source_sink", _dp),
        ("face_up", _ip), ("face_dn", _ip), ("gravdis", _dp),
        ("bnd_face", _ip), ("bnd_type", _ip), ("bnd_has_value", _ip),
        ("bnd_value", _dp), ("rho_bnd", _dp), ("vis_bnd", _dp),
        ("v_row_off", _ip), ("v_col_off", _ip), ("v_nint", _ip), ("v_trans_off", POINTER(c_longlong)),
        ("row_face", _ip), ("col_ext", _ip), ("trans", _dp),
    ]


def _load():
    if not _LIB.exists():
        import importlib.util

        spec = importlib.util.spec_from_file_location("tdycore_gb300_build",
                                                      _HERE.parent / "tdycore_gb300" / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build_oracle()
    lib = ctypes.CDLL(str(_LIB))
    lib.oracle_create.restype = c_void_p
    lib.oracle_create.argtypes = [POINTER(OracleInput)]
    lib.oracle_destroy.argtypes = [c_void_p]
    lib.oracle_max_threads.restype = c_int
    lib.oracle_pattern_nnz.restype = c_int
    lib.oracle_pattern_nnz.argtypes = [c_void_p]
    lib.oracle_pattern.argtypes = [c_void_p, _ip, _ip]
    lib.oracle_snes_presolve.argtypes = [c_void_p, _dp, c_double]
    lib.oracle_snes_function.argtypes = [c_void_p, _dp, _dp, _dp]
    lib.oracle_snes_jacobian.argtypes = [c_void_p, _dp, _dp, _dp]
    lib.oracle_ts_ifunction.argtypes = [c_void_p, _dp, _dp, _dp, _dp]
    lib.oracle_ts_ijacobian.argtypes = [c_void_p, _dp, _dp, c_double, _dp, _dp]
    lib.oracle_snes_function_jacobian_parallel.argtypes = [c_void_p, _dp, _dp, _dp, c_int]
    lib.oracle_snes_function_parallel.argtypes = [c_void_p, _dp, _dp, c_int]
    lib.oracle_get_state.argtypes = [c_void_p, _dp, _dp, _dp]
    lib.oracle_transient_variable.argtypes = [c_void_p, _dp, _dp, _dp]
    lib.oracle_tv_ifunction.argtypes = [c_void_p, _dp, _dp, _dp, _dp]
    lib.oracle_tv_ijacobian.argtypes = [c_void_p, _dp, c_double, _dp, _dp]
    lib.oracle_dae_ifunction.argtypes = [c_void_p, _dp, _dp, _dp, _dp]
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load()
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


class Oracle:
    """CPU restatement of the reference F/J over a setup view (dict)."""

    def __init__(self, view: dict):
        L = lib()
        self.view = view
        v = view
        self._arrays = {}

        def keep(name, dtype):
            a = np.ascontiguousarray(v[name], dtype=dtype)
            self._arrays[name] = a
            return a

        inp = OracleInput()
        inp.ncells, inp.nfaces, inp.nbnd, inp.nverts = v["ncells"], v["nfaces"], v["nbnd"], v["nverts"]
        inp.bc_type, inp.rho_type, inp.mu_type = v["bc_type"], v["rho_type"], v["mu_type"]
        inp.Pref = v["Pref"]
        for name in ("volume", "porosity", "Sr", "sat_param", "relperm_param", "source_sink", "gravdis",
                     "bnd_value", "rho_bnd", "vis_bnd", "trans"):
            setattr(inp, name, _p(keep(name, np.float64)))
        for name in ("sat_type", "relperm_type", "face_up", "face_dn", "bnd_face", "bnd_type", "bnd_has_value",
                     "v_row_off", "v_col_off", "v_nint", "row_face", "col_ext"):
            setattr(inp, name, _p(keep(name, np.int32), _ip))
        inp.v_trans_off = _p(keep("v_trans_off", np.int64), POINTER(c_longlong))
        self._ctx = L.oracle_create(ctypes.byref(inp))
        self.nc = v["ncells"]
        self.nnz = L.oracle_pattern_nnz(self._ctx)

    def __del__(self):
        try:
            lib().oracle_destroy(self._ctx)
        except Exception:
            pass

    def pattern(self):
        rp = np.empty(self.nc + 1, dtype=np.int32)
        ci = np.empty(self.nnz, dtype=np.int32)
        lib().oracle_pattern(self._ctx, _p(rp, _ip), _p(ci, _ip))
        return rp, ci

    def snes_presolve(self, U_prev, dt):
        u = np.ascontiguousarray(U_prev, dtype=np.float64)
        lib().oracle_snes_presolve(self._ctx, _p(u), dt)

    def snes_function(self, U, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty(self.nc)
        M = np.empty(self.nc) if with_mag else None
        lib().oracle_snes_function(self._ctx, _p(u), _p(R), _p(M) if with_mag else None)
        return (R, M) if with_mag else R

    def snes_jacobian(self, U, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        J = np.empty(self.nnz)
        M = np.empty(self.nnz) if with_mag else None
        lib().oracle_snes_jacobian(self._ctx, _p(u), _p(J), _p(M) if with_mag else None)
        return (J, M) if with_mag else J

    def ts_ifunction(self, U, Ut, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        ut = np.ascontiguousarray(Ut, dtype=np.float64)
        R = np.empty(self.nc)
        M = np.empty(self.nc) if with_mag else None
        lib().oracle_ts_ifunction(self._ctx, _p(u), _p(ut), _p(R), _p(M) if with_mag else None)
        return (R, M) if with_mag else R

    def ts_ijacobian(self, U, Ut, shift, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        ut = np.ascontiguousarray(Ut, dtype=np.float64)
        J = np.empty(self.nnz)
        M = np.empty(self.nnz) if with_mag else None
        lib().oracle_ts_ijacobian(self._ctx, _p(u), _p(ut), shift, _p(J), _p(M) if with_mag else None)
        return (J, M) if with_mag else J

    def transient_variable(self, U, with_derivative=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        C = np.empty(self.nc)
        dC = np.empty(self.nc) if with_derivative else None
        lib().oracle_transient_variable(self._ctx, _p(u), _p(C), _p(dC) if with_derivative else None)
        return (C, dC) if with_derivative else C

    def tv_ifunction(self, U, Mdot, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        md = np.ascontiguousarray(Mdot, dtype=np.float64)
        R = np.empty(self.nc)
        M = np.empty(self.nc) if with_mag else None
        lib().oracle_tv_ifunction(self._ctx, _p(u), _p(md), _p(R), _p(M) if with_mag else None)
        return (R, M) if with_mag else R

    def tv_ijacobian(self, U, shift, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        J = np.empty(self.nnz)
        M = np.empty(self.nnz) if with_mag else None
        lib().oracle_tv_ijacobian(self._ctx, _p(u), shift, _p(J), _p(M) if with_mag else None)
        return (J, M) if with_mag else J

    def dae_ifunction(self, U, Ut, with_mag=False):
        u = np.ascontiguousarray(U, dtype=np.float64)
        ut = np.ascontiguousarray(Ut, dtype=np.float64)
        R = np.empty(2 * self.nc)
        M = np.empty(2 * self.nc) if with_mag else None
        lib().oracle_dae_ifunction(self._ctx, _p(u), _p(ut), _p(R), _p(M) if with_mag else None)
        return (R, M) if with_mag else R

    def snes_function_parallel(self, U, nthreads=0):
        """The SNES residual with the vertex loop over colours on threads
        (equal to snes_function up to the summation order)."""
        u = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty(self.nc)
        lib().oracle_snes_function_parallel(self._ctx, _p(u), _p(R), nthreads)
        return R

    def snes_function_jacobian_parallel(self, U, nthreads=0):
        u = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty(self.nc)
        J = np.empty(self.nnz)
        lib().oracle_snes_function_jacobian_parallel(self._ctx, _p(u), _p(R), _p(J), nthreads)
        return R, J

    def state(self):
        S, rho, kr = np.empty(self.nc), np.empty(self.nc), np.empty(self.nc)
        lib().oracle_get_state(self._ctx, _p(S), _p(rho), _p(kr))
        return S, rho, kr


def max_threads() -> int:
    return lib().oracle_max_threads()
