"""Newton driver used by the golden regression tests.

Restates the defaults of PETSc's SNESNEWTONLS (pinned PETSc v3.17.3) that the
reference's regression runs use: full Newton step, backtracking line search
accepting lambda when ||F(x - lambda y)||^2 <= (1 - 2*1e-4*lambda) ||F(x)||^2,
and SNESConvergedDefault with rtol = stol = 1e-8 (relative residual, or step
norm below stol * ||x||).  Linear solves are direct (-pc_type lu).
``F`` and ``J`` are callables returning the residual and the CSR values.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def newton(F, J, x, rowptr, colidx, rtol=1e-8, stol=1e-8, maxit=50):
    n = x.size
    f = F(x)
    fnorm = np.linalg.norm(f)
    ttol = fnorm * rtol
    for it in range(maxit):
        A = sp.csr_matrix((J(x), colidx, rowptr), shape=(n, n)).tocsc()
        y = spla.spsolve(A, f)
        lam = 1.0
        while True:
            xn = x - lam * y
            fn = F(xn)
            fnn = np.linalg.norm(fn)
            if fnn * fnn <= (1.0 - 2.0e-4 * lam) * fnorm * fnorm or lam < 1e-10:
                break
            lam *= 0.5
        x, f, fnorm = xn, fn, fnn
        if fnorm < ttol or lam * np.linalg.norm(y) < stol * np.linalg.norm(x):
            return x, it + 1
    raise RuntimeError("Newton did not converge")


def snes_steps(o, U, dt, nsteps):
    """Backward Euler with the SNES form (TDyPreSolveSNESSolver + SNESSolve)."""
    rp, ci = o.pattern()
    for _ in range(nsteps):
        o.snes_presolve(U, dt)
        U, _ = newton(o.snes_function, o.snes_jacobian, U.copy(), rp, ci)
    return U


def ts_beuler_steps(o, U, dt, nsteps):
    """TSBEULER with IFunction/IJacobian: F(U, (U - U_n)/dt) = 0, shift = 1/dt."""
    rp, ci = o.pattern()
    for _ in range(nsteps):
        Un = U.copy()
        U, _ = newton(lambda x: o.ts_ifunction(x, (x - Un) / dt),
                      lambda x: o.ts_ijacobian(x, (x - Un) / dt, 1.0 / dt), U.copy(), rp, ci)
    return U
