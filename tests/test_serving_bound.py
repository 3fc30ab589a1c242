"""The ideal fluid scheduler behind the serving sweep's bound (host logic,
no GPU): known completion times on small cases, work conservation, and the
bound computed from isolated solves."""
import numpy as np
import pytest

from fastqsl_gb300.serving import QRequest, fluid_schedule, ideal_bound


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


def test_bench_request_mix_is_beyond_the_serving_bar_for_any_scheduler():
    """The serving sweep's request stream (96 requests, 10^4-4x10^6 seeds
    log-uniform, seed 7) under a linear cost model: isolated time = Q-pixels x
    a per-tolerance cost, at least 3 ms (small requests cannot fill the GPU).
    At 80 % load even the ideal preemptive SRPT scheduler's p99 is far above
    2x isolated: the largest requests queue behind each other whatever the
    order.  At 50 % load it is lower but still above 2x."""
    from fastqsl_gb300.serving import make_requests
    shape, names = (384, 384, 256), [f"f{k}" for k in range(8)]
    burst = make_requests(shape, names, 96, None, seed=7)
    cost = {1e-3: 0.6, 1e-4: 1.0, 1e-5: 1.7}
    rate_px = 80e6  # Q-pixels/s of the saturated GPU at tol 1e-4
    iso = {r.rid: max(r.qpixels / rate_px * cost[r.tol], 0.003) for r in burst}
    span = sum(r.qpixels / rate_px * cost[r.tol] for r in burst)  # saturated: the work itself
    p99 = {}
    for f in (0.5, 0.8):
        reqs = make_requests(shape, names, 96, f * 96 / span, seed=7)
        p99[f] = ideal_bound(reqs, iso, span, policies=("srpt",))["srpt"][1]
    assert p99[0.8] > 4.0 and p99[0.5] > 2.0 and p99[0.8] > p99[0.5]
