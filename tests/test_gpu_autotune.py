"""The launch-configuration tuner measures every candidate (seed tile,
register budget, static lockstep or work queue with its refill size) and
applies the fastest; the tuned plan's Q equals an untuned plan's to
rounding."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_tune_plan(cuda):
    from fastqsl_gb300 import api, autotune, params as P, synthetic as S
    spec = S.charges_random(4, (64, 64, 48), 8)
    B = S.make_field(spec)
    fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout="h4b")
    n0 = n1 = 34
    xs, ys, zs = api.plane_seed_grid(14.0, 47.0, n1, 14.0, 47.0, n0, [5.0, 9.0, 13.0])
    prm = P.absolute_rkf45()
    plan = api.QMapPlan(n0, n1, 3)
    q0 = plan.run(fs, xs, ys, zs, prm, s_len=0.25).cpu().numpy()
    res = autotune.tune_plan(plan, fs, xs, ys, zs, prm, s_len=0.25, sample_planes=2, use_cache=False)
    # every tile x budget in static lockstep, then the work queue at each
    # refill size on the best of those
    assert len(res["table"]) == len(autotune.TILES) * len(autotune.OCCUPANCIES) + len(autotune.QUEUE_CHUNKS)
    assert res["ms"] == min(res["table"].values())
    assert res["schedule"] in ("static", "queue") and plan.schedule == res["schedule"]
    if res["schedule"] == "queue":
        assert plan.chunk == res["chunk"] in autotune.QUEUE_CHUNKS
    q1 = plan.run(fs, xs, ys, zs, prm, s_len=0.25).cpu().numpy()
    assert (np.isnan(q0) == np.isnan(q1)).mean() >= 0.99
    ok = ~np.isnan(q0) & ~np.isnan(q1)
    assert np.median(np.abs(np.log10(q0[ok]) - np.log10(q1[ok]))) <= 1e-5
