"""Time integrator, Newton driver, regression output and PETSc-binary I/O.

The two reference regression runs that go through the driver
(demo/richards/richards.cfg [richards-driver-snes-prob1] and
demo/transient/transient_snes_mpfaof90.cfg [transient-snes-mpfaof90-tdydriver])
are reproduced at the reference harness's tolerance (1e-12 relative), once
with the oracle's residual/Jacobian on the CPU and once with the GPU path.
The written regression file must parse to the gold values.
"""
import base64
import json
from pathlib import Path

import numpy as np
import pytest

import tdycore_gb300 as T
from tdycore_gb300 import driver as D
from tdycore_gb300.workloads import box_column
from oracle import Oracle

GOLDEN = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())
GOLD = GOLDEN["cases"]
RTOL = 1.0e-12


def parse_regression(text):
    out = {"sampled": {}}
    for line in text.splitlines():
        line = line.strip()
        if ":" not in line or line.startswith("--"):
            continue
        k, v = [s.strip() for s in line.split(":", 1)]
        if k in ("Max", "Min", "Mean"):
            out[k.lower()] = float(v)
        else:
            out["sampled"][k] = float(v)
    return out


def check_against_gold(name, got):
    g = GOLD[name]
    for k in ("max", "min", "mean"):
        assert abs(got[k] - g[k]) <= RTOL * abs(g[k]), (name, k, got[k], g[k])
    assert set(got["sampled"]) == set(g["sampled"]), (got["sampled"], g["sampled"])
    for idx, val in g["sampled"].items():
        assert abs(got["sampled"][idx] - val) <= RTOL * abs(val), (name, idx, got["sampled"][idx], val)


class OracleTDy:
    """The TDy methods the driver calls, served by the oracle (CPU) over the
    host setup of a real handle; regression output goes through the handle."""

    def __init__(self, t):
        self.t = t
        self.o = Oracle(t.setup_view())
        self.ncells = t.ncells
        self.rowptr, self.colidx = t.rowptr, t.colidx
        self.dt = None
        self.prev = None

    def set_dtime(self, dt):
        self.dt = dt

    def set_previous_solution(self, U):
        self.prev = np.array(U, dtype=np.float64)

    def presolve_current(self):
        self.o.snes_presolve(self.prev, self.dt)

    def post_solve(self, U):
        self.set_previous_solution(U)

    def snes_function(self, U):
        return self.o.snes_function(U)

    def snes_jacobian(self, U):
        return self.o.snes_jacobian(U)

    def ifunction(self, time, U, Ut):
        return self.o.ts_ifunction(U, Ut)

    def ijacobian(self, time, U, Ut, shift):
        return self.o.ts_ijacobian(U, Ut, shift)

    def output_regression(self, U):
        self.t.output_regression(U)


def prob1_case(tmp_path, name):
    """demo/richards/richards.cfg [richards-driver-snes-prob1]: 2x2x2 box on
    the unit cube, exponential density, properties from the option defaults,
    IC from the PETSc binary file."""
    vec = tmp_path / "prob1_ic.vec"
    vec.write_bytes(base64.b64decode(GOLDEN["richards_prob1_ic_petsc_binary_b64"]))
    T.options_clear()
    T.options_insert(f"-tdy_water_density exponential -tdy_regression_test "
                     f"-tdy_regression_test_num_cells_per_process 2 -tdy_regression_test_filename {tmp_path / name} "
                     f"-tdy_final_time 3.1536e3 -tdy_dt_max 600. -tdy_dt_growth_factor 1.5 "
                     f"-tdy_init_file {vec} -tdy_time_integration_method SNES -tdy_dt_init 0.1")
    t = T.create_richards_mpfao()
    t.set_box_mesh(2, 2, 2, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    t.set_from_options()
    return t


def tdydriver_case(tmp_path, name):
    """transient_snes_mpfaof90 -use_tdydriver: the 1x1x15 column of the demo,
    ten RunToTime(1800 * step) calls with the time step reset to 1800 s."""
    T.options_clear()
    T.options_insert(f"-tdy_regression_test -tdy_regression_test_num_cells_per_process 2 "
                     f"-tdy_regression_test_filename {tmp_path / name}")
    return box_column(1, 1, 15)


def run_prob1(handle, t):
    ti = D.TimeIntegrator(handle)
    ti.set_solution(D.initial_condition(t.ncells))
    ti.run_to_time(ti.final_time)
    ti.output_regression()
    return ti


def run_tdydriver(handle):
    ti = D.TimeIntegrator(handle)
    ti.set_solution(np.full(handle.ncells, 102325.0))
    for step in range(1, 11):
        ti.set_time_step(1800.0)
        ti.run_to_time(1800.0 * step)
    ti.output_regression()
    return ti


# ---------------------------------------------------------------------------
# CPU


def test_petsc_binary_vec_reader_and_writer(tmp_path):
    raw = base64.b64decode(GOLDEN["richards_prob1_ic_petsc_binary_b64"])
    u = D.read_petsc_vec(raw)
    assert np.array_equal(u, np.array(GOLDEN["richards_prob1_ic"]))
    p = tmp_path / "u.vec"
    D.write_petsc_vec(p, u)
    assert p.read_bytes() == raw
    with pytest.raises(ValueError):
        D.read_petsc_vec(raw[:20])
    with pytest.raises(ValueError):
        D.read_petsc_vec(b"\x00" * 16)


def test_options_queries():
    T.options_clear()
    T.options_insert("-tdy_final_time 3.5e3 -tdy_dt_max -2 -flag -tdy_init_file a.vec -n 7")
    assert T.options_get_real("-tdy_final_time") == 3.5e3
    assert T.options_get_real("-tdy_dt_max") == -2.0
    assert T.options_get_real("-tdy_missing", 1.25) == 1.25
    assert T.options_get_string("-tdy_init_file") == "a.vec"
    assert T.options_get_int("-n") == 7
    assert T.options_has_name("-flag") and not T.options_has_name("-nope")
    with pytest.raises(T.TDyError):
        T.options_get_real("-tdy_init_file")
    T.options_clear()


def test_time_step_logic_matches_reference_rules():
    """dt growth, dt_max cap and the shortened last step (src/tdyti.c:72-90)."""

    class Fake:
        ncells = 1
        rowptr = np.array([0, 1])
        colidx = np.array([0])

        def set_dtime(self, dt):
            self.dt = dt

        def set_previous_solution(self, U):
            pass

        def presolve_current(self):
            pass

        def post_solve(self, U):
            pass

        def snes_function(self, U):
            return U - 1.0

        def snes_jacobian(self, U):
            return np.ones(1)

    T.options_clear()
    T.options_insert("-tdy_dt_init 0.1 -tdy_dt_growth_factor 1.5 -tdy_dt_max 600 -tdy_final_time 3153.6")
    ti = D.TimeIntegrator(Fake())
    T.options_clear()
    ti.set_solution(np.zeros(1))
    ti.run_to_time(ti.final_time)
    dts = [h[2] for h in ti.history]
    assert dts[0] == 0.1 and abs(dts[1] - 0.15) < 1e-15
    assert max(dts) == 600.0
    assert abs(sum(dts) - 3153.6) < 1e-9 and abs(ti.time - 3153.6) < 1e-9
    # geometric growth until the cap, then the remainder
    for a, b in zip(dts[:-1], dts[1:-1]):
        assert abs(b - min(a * 1.5, 600.0)) <= 1e-12 * b


def test_newton_reasons():
    s = D.SNESNewtonLS()
    rp, ci = np.array([0, 1]), np.array([0])
    r = s.solve(lambda x: x * x - 4.0, lambda x: 2.0 * x, np.array([3.0]), rp, ci)
    assert r.reason in (D.CONVERGED_FNORM_RELATIVE, D.CONVERGED_SNORM_RELATIVE) and abs(r.x[0] - 2.0) < 1e-8
    r = s.solve(lambda x: x * x + 1.0, lambda x: 2.0 * x, np.array([0.5]), rp, ci)
    assert r.reason < 0


def test_driver_goldens_oracle(tmp_path):
    t = prob1_case(tmp_path, "prob1")
    t.setup(host_only=True)
    run_prob1(OracleTDy(t), t)
    check_against_gold("richards-driver-snes-prob1", parse_regression((tmp_path / "prob1.regression").read_text()))

    t = tdydriver_case(tmp_path, "tdydriver")
    t.setup(host_only=True)
    run_tdydriver(OracleTDy(t))
    check_against_gold("transient-snes-mpfaof90-tdydriver",
                       parse_regression((tmp_path / "tdydriver.regression").read_text()))
    T.options_clear()


def test_regression_file_format(tmp_path):
    """Same layout as the gold files: header, Max/Min/Mean, sampled cells."""
    T.options_clear()
    T.options_insert(f"-tdy_regression_test -tdy_regression_test_filename {tmp_path / 'fmt'}")
    t = box_column(1, 1, 15)
    t.setup(host_only=True)
    U = 1e5 + np.arange(15.0)
    t.output_regression(U)
    text = (tmp_path / "fmt.regression").read_text()
    gold = GOLDEN["gold_text"]["transient-snes-mpfaof90-tdydriver"]
    assert [ln[:10] for ln in text.splitlines()] == [ln[:10] for ln in gold.splitlines()]
    assert text.splitlines()[1] == "      Max:   1.0001400000000e+05"
    assert parse_regression(text)["sampled"] == {"0": 1e5, "7": 1e5 + 7}
    T.options_clear()
    # -tdy_regression_test without a filename is an error at TDySetup
    T.options_insert("-tdy_regression_test")
    t = box_column(1, 1, 3)
    with pytest.raises(T.TDyError):
        t.setup(host_only=True)
    T.options_clear()


# ---------------------------------------------------------------------------
# GPU


@pytest.mark.gpu
def test_driver_goldens_gpu(tmp_path):
    t = prob1_case(tmp_path, "prob1")
    t.setup()
    run_prob1(t, t)
    check_against_gold("richards-driver-snes-prob1", parse_regression((tmp_path / "prob1.regression").read_text()))

    t = tdydriver_case(tmp_path, "tdydriver")
    t.setup()
    run_tdydriver(t)
    check_against_gold("transient-snes-mpfaof90-tdydriver",
                       parse_regression((tmp_path / "tdydriver.regression").read_text()))
    T.options_clear()


@pytest.mark.gpu
def test_infiltration_newton_gpu_matches_oracle():
    """The 10x10x10 box started 60 kPa below hydrostatic (unsaturated): the
    same host Newton around the GPU residual/Jacobian and around the oracle's
    takes the same iterations on the steps that do real work and reaches the
    same pressures."""
    from tdycore_gb300.workloads import hydrostatic_box

    T.options_clear()
    t, U0, _ = hydrostatic_box()
    t.setup()
    t.set_dtime(1800.0)
    o = Oracle(t.setup_view())
    Ug, Uc = U0 - 60000.0, U0 - 60000.0
    for step in range(3):
        t.presolve(Ug)
        o.snes_presolve(Uc, 1800.0)
        rg = D.SNESNewtonLS().solve(t.snes_function, t.snes_jacobian, Ug.copy(), t.rowptr, t.colidx)
        rc = D.SNESNewtonLS().solve(o.snes_function, o.snes_jacobian, Uc.copy(), t.rowptr, t.colidx)
        assert rg.reason > 0 and rc.reason > 0
        if step == 0:
            assert rg.iterations == rc.iterations >= 5
        Ug, Uc = rg.x, rc.x
        assert np.max(np.abs(Ug - Uc) / np.abs(Uc)) < 1e-12
    t.destroy()
