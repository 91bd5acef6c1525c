"""Continuous-batching server: admission by slots and HBM budget in arrival
order (CPU, with a stand-in runner), the summary's counting rules (CPU), and
on the GPU each request's result the same alone and in a mix, every step
converged."""
import threading
import time

import numpy as np
import pytest

from tdycore_gb300 import serving as S


def _requests(n, sizes, gaps):
    t, out = 0.0, []
    for i in range(n):
        t += gaps[i]
        out.append(S.Request(rid=i, arrival_s=t, nx=1, ny=1, nz=int(sizes[i]), dz=0.1, k=1e-12, porosity=0.3,
                             alpha=1e-4, m=0.4, forcing=np.zeros(2)))
    return out


def test_admission_respects_slots_budget_and_order():
    n = 24
    rng = np.random.default_rng(0)
    reqs = _requests(n, rng.integers(1, 10, n), rng.uniform(0.0, 0.004, n))
    live, peak, lock = [0], [0], threading.Lock()

    def runner(group, finished):
        (r,) = group
        with lock:
            live[0] += 1
            peak[0] = max(peak[0], live[0])
        time.sleep(0.01 + 0.002 * r.nz)
        with lock:
            live[0] -= 1

    fp = lambda nc: 10 * nc  # noqa: E731  budget units per cell
    srv = S.Server(slots=4, hbm_budget_bytes=100, runner=runner, footprint=fp, cohort=1)
    done = srv.run(reqs)
    assert all(r.error is None for r in done)
    assert peak[0] <= 4 and srv.peak_running <= 4
    assert srv.peak_in_use <= 100
    admitted = [r.admitted_s for r in sorted(done, key=lambda r: r.arrival_s)]
    assert admitted == sorted(admitted), "admission follows arrival order"
    assert all(r.admitted_s >= r.arrival_s - 1e-9 and r.finished_s > r.admitted_s for r in done)
    with pytest.raises(ValueError):
        S.Server(slots=2, hbm_budget_bytes=5, runner=runner, footprint=fp, cohort=1).run(_requests(1, [1], [0.0]))


def test_cohorts_are_consecutive_same_class_and_within_budget():
    """Requests that have arrived and wait when a slot frees up form one
    cohort: consecutive in arrival order, of one size class (large requests
    alone), at most ``cohort`` of them, within the HBM budget."""
    reqs = _requests(30, [5] * 30, [0.0] * 30)
    for r in reqs[10:13]:
        r.nx, r.ny, r.nz = 64, 64, 50  # large
    seen, lock = [], threading.Lock()

    def runner(group, finished):
        with lock:
            seen.append([r.rid for r in group])
        for r in group:
            finished(r)
        time.sleep(0.02)

    fp = lambda nc: nc  # noqa: E731
    srv = S.Server(slots=1, hbm_budget_bytes=1e6, runner=runner, footprint=fp, cohort=4)
    done = srv.run(reqs)
    assert all(r.error is None and r.finished_s >= r.admitted_s for r in done)
    flat = [rid for g in seen for rid in g]
    assert flat == sorted(flat) == list(range(30)), "every request once, in arrival order"
    for g in seen:
        assert len(g) <= 4
        cls = {S.size_class(reqs[rid]) for rid in g}
        assert len(cls) == 1
        if cls == {1}:
            assert len(g) == 1
    assert max(len(g) for g in seen) == 4 and srv.cohorts == [len(g) for g in seen]


def test_request_generator_statistics():
    reqs = S.make_requests(400, rate_per_s=50.0, nsteps=24, seed=1)
    gaps = np.diff([0.0] + [r.arrival_s for r in reqs])
    assert abs(gaps.mean() - 1 / 50.0) < 0.25 / 50.0
    large = [r for r in reqs if (r.nx, r.ny, r.nz) == (64, 64, 50)]
    assert 5 <= len(large) <= 40
    small = [r for r in reqs if r.nz != 50 or r.nx != 64]
    assert all(1 <= r.nx <= 8 and 1 <= r.ny <= 8 and 10 <= r.nz <= 100 for r in small)
    f = np.concatenate([r.forcing for r in reqs])
    assert abs(f.std() - 1e-7) < 1e-8


def test_summary_counts_converged_solves_and_completed_requests():
    """A request ends at its first unconverged step (reported as its error);
    latency percentiles cover completed requests, solves/s converged solves."""
    reqs = _requests(3, [4, 4, 4], [0.0, 0.0, 0.0])
    for r in reqs:
        r.forcing = np.zeros(3)
        r.admitted_s, r.finished_s = r.arrival_s, r.arrival_s + 2.0
    reqs[0].rel_residual, reqs[0].converged_steps = [1e-9, 1e-9, 1e-9], 3
    reqs[1].rel_residual, reqs[1].converged_steps = [1e-9, 1e-9, 1e-9], 3
    reqs[2].rel_residual, reqs[2].converged_steps = [1e-9, 0.5], 1
    reqs[2].error = "step 2 did not converge (relative residual 5.0e-01)"
    reqs[2].finished_s = reqs[2].arrival_s + 9.0
    out = S.summary(reqs, wall_s=7.0)
    assert out["errors"] == 1 and out["converged_solves"] == 7
    assert out["solves_attempted"] == 8 and out["solves_requested"] == 9
    assert out["solves_per_s"] == 1.0
    assert out["p99_latency_s"] <= 2.0 + 1e-12


@pytest.mark.gpu
def test_same_result_alone_and_in_the_mix():
    """Requests served in cohorts (one batched handle each) give every request
    the bits it gets alone."""
    reqs = S.make_requests(8, rate_per_s=400.0, nsteps=3, large_fraction=0.0, seed=5)
    srv = S.Server(slots=4, cohort=4)
    mix = srv.run(reqs)
    assert all(r.error is None for r in mix), [r.error for r in mix]
    assert all(r.converged_steps + r.step_test_steps == 3 for r in mix)
    for k in (0, 5):
        alone = S.make_requests(8, rate_per_s=400.0, nsteps=3, large_fraction=0.0, seed=5)[k]
        S.run_request(alone)
        assert np.array_equal(alone.U_final, mix[k].U_final)
        assert alone.newton_its == mix[k].newton_its


@pytest.mark.gpu
def test_concurrent_requests_with_overlapping_setup_and_teardown():
    """24 requests arriving at once on 16 slots: while some requests iterate
    (and build their inner-solve graphs), others set up or destroy their
    handles.  No request may fail for any reason but a step that does not
    converge, and a request's result is the same as when it runs alone."""
    reqs = S.make_requests(24, rate_per_s=5000.0, nsteps=2, large_fraction=0.0, seed=11)
    srv = S.Server(slots=16, cohort=1)
    done = srv.run(reqs)
    assert srv.peak_running >= 16
    bad = [r.error for r in done if r.error is not None and "did not converge" not in r.error]
    assert not bad, bad
    assert sum(r.converged_steps + r.step_test_steps for r in done) >= 40
    for k in (3, 17):
        alone = S.make_requests(24, rate_per_s=5000.0, nsteps=2, large_fraction=0.0, seed=11)[k]
        S.run_request(alone)
        assert alone.error == done[k].error
        assert np.array_equal(alone.U_final, done[k].U_final)
