"""The ideal fluid scheduler behind the serving sweep's bounds (host logic,
no GPU): known completion times on small cases, work conservation, the
bound computed from isolated solves, and the smallest worst-request ratio
any schedule reaches (deadline feasibility as a maximum flow)."""
import numpy as np
import pytest

from fastqsl_gb300.serving import QRequest, fluid_schedule, ideal_bound, min_max_stretch, _deadlines_feasible


def test_single_job_runs_at_its_cap():
    assert fluid_schedule([0.0], [2.0], [1.0]) == pytest.approx([2.0])
    assert fluid_schedule([1.0], [2.0], [0.5], capacity=4.0) == pytest.approx([5.0])


def test_two_equal_jobs_per_policy():
    a, w, c = [0.0, 0.0], [1.0, 1.0], [1.0, 1.0]
    assert sorted(fluid_schedule(a, w, c, policy="srpt")) == pytest.approx([1.0, 2.0])
    assert fluid_schedule(a, w, c, policy="ps") == pytest.approx([2.0, 2.0])
    assert fluid_schedule(a, w, c, policy="fcfs") == pytest.approx([1.0, 2.0])


def test_srpt_preempts_a_long_job():
    # a long job at t=0, a short one at t=1: SRPT runs the short one at once
    done = fluid_schedule([0.0, 1.0], [10.0, 1.0], [1.0, 1.0], policy="srpt")
    assert done == pytest.approx([11.0, 2.0])
    done = fluid_schedule([0.0, 1.0], [10.0, 1.0], [1.0, 1.0], policy="fcfs")
    assert done == pytest.approx([10.0, 11.0])
    # PS: both at rate 1/2 from t=1; the short one ends at 3, the long at 11
    done = fluid_schedule([0.0, 1.0], [10.0, 1.0], [1.0, 1.0], policy="ps")
    assert done == pytest.approx([11.0, 3.0])


def test_caps_leave_room_for_others():
    # two jobs capped at 0.4 of a unit capacity run side by side at their caps
    done = fluid_schedule([0.0, 0.0], [0.4, 0.8], [0.4, 0.4], policy="srpt")
    assert done == pytest.approx([1.0, 2.0])
    # water-filling: a capped job takes its cap, the other the rest
    done = fluid_schedule([0.0, 0.0], [0.2, 3.0], [0.2, 1.0], policy="ps")
    assert done == pytest.approx([1.0, 1.0 + (3.0 - 0.8) / 1.0])


def test_work_conservation_on_a_random_stream():
    rng = np.random.default_rng(3)
    n = 60
    a = np.cumsum(rng.exponential(1.0, n))
    w = np.exp(rng.uniform(np.log(0.05), np.log(3.0), n))
    for pol in ("srpt", "ps", "fcfs"):
        done = fluid_schedule(a, w, np.ones(n), policy=pol)
        assert np.all(done >= a + w - 1e-9)
        # a single unit-rate server: the last completion is the same under
        # every work-conserving policy
        assert done.max() == pytest.approx(fluid_schedule(a, w, np.ones(n), policy="fcfs").max())
    # SRPT never has a larger mean response time than PS or FCFS
    mean = {p: np.mean(fluid_schedule(a, w, np.ones(n), policy=p) - a) for p in ("srpt", "ps", "fcfs")}
    assert mean["srpt"] <= mean["ps"] + 1e-9 and mean["srpt"] <= mean["fcfs"] + 1e-9


def test_rejects_bad_inputs():
    with pytest.raises(ValueError):
        fluid_schedule([0.0], [1.0], [0.0])
    with pytest.raises(ValueError):
        fluid_schedule([0.0], [1.0], [1.0], policy="lifo")
    with pytest.raises(ValueError):
        fluid_schedule([], [], [], policy="lifo")
    with pytest.raises(ValueError):
        fluid_schedule([0.0, 1.0], [1.0], [1.0, 1.0])
    assert len(fluid_schedule([], [], [])) == 0


def test_ideal_bound_from_isolated_solves():
    # two requests that fill the GPU and one small one, all at one tolerance
    reqs = [QRequest(rid=0, field="f", n0=102, n1=102, arrival=0.0),      # 10^4 Q-pixels
            QRequest(rid=1, field="f", n0=102, n1=102, arrival=0.0),
            QRequest(rid=2, field="f", n0=12, n1=12, arrival=0.5)]         # 100 Q-pixels
    iso = {0: 1.0, 1: 1.0, 2: 0.1}     # the small one cannot fill the GPU: rate 0.1 of it
    # saturated span 2.01: the capacity is the work of the set (2.01) over it = 1
    b = ideal_bound(reqs, iso, 2.01)
    # SRPT: the small request runs at its cap beside the first large one and
    # finishes in its isolated time (ratio 1); the first large one lost 0.01
    # of work to it (1.01), the second waited for the first (2.01)
    assert b["srpt"][1] == pytest.approx(np.percentile([1.01, 2.01, 1.0], 99), rel=1e-9)
    assert b["ps"][0] >= 1.0


def test_deadline_feasibility_with_caps():
    """Two jobs at t = 0 on a unit-capacity server: A (work 1, at most rate
    1) and B (work 1, at most rate 1/2).  Both can end by t = 2 (each at
    rate 1/2 throughout), although earliest-deadline-first, which gives A the
    whole server first, misses B's deadline; no schedule ends A by 1.9 and B
    by 2."""
    a, w, c = np.array([0.0, 0.0]), np.array([1.0, 1.0]), np.array([1.0, 0.5])
    assert _deadlines_feasible(a, w, c, np.array([2.0, 2.0]), 1.0)
    assert not _deadlines_feasible(a, w, c, np.array([1.9, 2.0]), 1.0)
    assert not _deadlines_feasible(a, w, c, np.array([0.9, 5.0]), 1.0)  # A alone needs 1


def test_min_max_stretch_known_value():
    # the two jobs above, isolated times 1 and 2: with ratio s, A must end by
    # s and B by 2s; B gets min(s/2, s - 1) before s and s/2 after, so the
    # smallest feasible s is 4/3
    a, w, c = np.array([0.0, 0.0]), np.array([1.0, 1.0]), np.array([1.0, 0.5])
    assert min_max_stretch(a, w, c, w / c, 1.0) == pytest.approx(4.0 / 3.0, rel=2e-3)
    # jobs that never overlap: every ratio is 1
    assert min_max_stretch([0.0, 5.0], [1.0, 1.0], [1.0, 1.0], [1.0, 1.0], 1.0) == 1.0


def test_min_max_stretch_below_every_policy():
    """No schedule beats the bound, and the fluid policies' worst ratios are
    schedules, so the bound lies at or below each of them."""
    rng = np.random.default_rng(4)
    n = 200
    a = np.cumsum(rng.exponential(1.0, n))
    w = np.exp(rng.uniform(np.log(0.05), np.log(3.0), n))
    c = np.minimum(1.0, w / 0.3)
    iso = w / c
    mm = min_max_stretch(a, w, c, iso, 1.25)
    assert mm >= 1.0
    for pol in ("srpt", "ps", "fcfs"):
        worst = np.max((fluid_schedule(a, w, c, 1.25, pol) - a) / iso)
        assert mm <= worst * (1 + 1e-3)
    # the deadlines at the bound are feasible, 1 % below it they are not
    assert _deadlines_feasible(a, w, c, a + mm * (1 + 2e-3) * iso, 1.25)
    assert not _deadlines_feasible(a, w, c, a + mm * 0.99 * iso, 1.25)


def _cost_model_stream(count, fraction, seeds_range):
    """The serving sweep's request stream (seed 7) under a linear cost model:
    isolated time = Q-pixels x a per-tolerance cost, at least 3 ms (small
    requests cannot fill the GPU); the saturated span is the work itself."""
    from fastqsl_gb300.serving import make_requests
    shape, names = (384, 384, 256), [f"f{k}" for k in range(8)]
    burst = make_requests(shape, names, count, None, seed=7, seeds_range=seeds_range)
    cost = {1e-3: 0.6, 1e-4: 1.0, 1e-5: 1.7}
    rate_px = 80e6  # Q-pixels/s of the saturated GPU at tol 1e-4
    iso = {r.rid: max(r.qpixels / rate_px * cost[r.tol], 0.003) for r in burst}
    span = sum(r.qpixels / rate_px * cost[r.tol] for r in burst)
    reqs = make_requests(shape, names, count, fraction * count / span, seed=7, seeds_range=seeds_range)
    return reqs, iso, span


def test_wide_request_mix_is_beyond_the_serving_bar_for_ideal_schedulers():
    """The serving configuration's mix (10^4-4x10^6 seeds, log-uniform) at
    80 % load under the cost model: the ideal preemptive SRPT and processor-
    sharing schedulers' p99 and the smallest worst-request ratio of any
    schedule all lie far above 2x isolated: the largest requests fill the GPU
    and queue behind each other whatever the order."""
    reqs, iso, span = _cost_model_stream(512, 0.8, (1e4, 4e6))
    b = ideal_bound(reqs, iso, span, min_max=True)
    assert b["srpt"][1] > 4.0 and b["ps"][1] > 4.0 and b["min_max"] > 4.0


def test_small_request_mix_is_within_the_serving_bar_for_an_ideal_scheduler():
    """The bench's second mix (10^4-3x10^4 seeds): no request fills the GPU
    alone, several run side by side at full speed, and the ideal SRPT
    scheduler's p99 at 80 % load stays under 2x isolated, so on this mix the
    bar is a test of the server's scheduling."""
    reqs, iso, span = _cost_model_stream(512, 0.8, (1e4, 3e4))
    b = ideal_bound(reqs, iso, span)
    assert b["srpt"][1] < 2.0
