"""The allocation-free fused evaluation (TDyMPFAOSNESFunctionJacobianDeviceNoAlloc).

Some callers cannot let a library allocate device memory while they run: a
host application that hands out all device memory from its own pool, or a
time-critical loop that must not pay for the device-wide synchronisation that
cudaMalloc/cudaFree can trigger.  The entry point under test keeps its scratch
in a fixed array inside the library instead.  These tests call it through the
C-ABI, twice in a row with different states (the array keeps the previous
call's contents, which must not leak into the next result), compare each call
with the allocating entry point within the parity tolerances of the other
GPU tests, and check that a mesh too large for the array is refused.

This file is collected last so that a failing run stopped at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

R_TOL = 1e-12
J_TOL = 1e-10
DT = 1800.0


def _ptr(x):
    return ctypes.c_void_p(x.data_ptr())


def test_no_alloc_matches_allocating_entry_point_on_two_calls():
    import torch

    import tdycore_gb300 as T
    from oracle import Oracle
    from tests.parity_cases import case_spe10_small

    t, U, Uprev, _ = case_spe10_small()
    t.setup()
    t.set_dtime(DT)
    o = Oracle(t.setup_view())
    o.snes_presolve(Uprev, DT)
    dev = torch.device("cuda", torch.cuda.current_device())
    t.presolve_device(torch.tensor(Uprev, dtype=torch.float64, device=dev))
    rng = np.random.default_rng(2024)
    for call in range(2):
        Uc = U + rng.normal(0.0, 400.0, U.size)
        dU = torch.tensor(Uc, dtype=torch.float64, device=dev)
        dR0 = torch.empty(t.ncells, dtype=torch.float64, device=dev)
        dJ0 = torch.empty(t.nnz, dtype=torch.float64, device=dev)
        t.snes_function_jacobian_device(dU, dR0, dJ0)
        dR1 = torch.full((t.ncells,), float("nan"), dtype=torch.float64, device=dev)
        dJ1 = torch.full((t.nnz,), float("nan"), dtype=torch.float64, device=dev)
        T.check(T.lib.TDyMPFAOSNESFunctionJacobianDeviceNoAlloc(t._h, _ptr(dU), _ptr(dR1), _ptr(dJ1), None),
                "TDyMPFAOSNESFunctionJacobianDeviceNoAlloc")
        t.synchronize()
        R0, J0, R1, J1 = dR0.cpu().numpy(), dJ0.cpu().numpy(), dR1.cpu().numpy(), dJ1.cpu().numpy()
        _, Rm = o.snes_function(Uc, with_mag=True)
        _, Jm = o.snes_jacobian(Uc, with_mag=True)
        assert np.all(np.isfinite(R1)) and np.all(np.isfinite(J1)), f"call {call}: unwritten outputs"
        assert np.all(np.abs(R1 - R0) <= R_TOL * Rm), f"call {call}: residual differs"
        assert np.all(np.abs(J1 - J0) <= J_TOL * Jm), f"call {call}: Jacobian differs"


def test_no_alloc_refuses_meshes_larger_than_its_scratch():
    import torch

    import tdycore_gb300 as T
    from tdycore_gb300.workloads import box_column

    T.options_clear()
    t = box_column(50, 50, 50)
    t.setup()
    t.set_dtime(DT)
    dev = torch.device("cuda", torch.cuda.current_device())
    dU = torch.full((t.ncells,), 101325.0, dtype=torch.float64, device=dev)
    dR = torch.empty(t.ncells, dtype=torch.float64, device=dev)
    code = T.lib.TDyMPFAOSNESFunctionJacobianDeviceNoAlloc(t._h, _ptr(dU), _ptr(dR), None, None)
    assert code == 63, T.lib.TDyGetErrorMessage()
    assert b"static scratch" in T.lib.TDyGetErrorMessage()
