"""Batched uneven solves (many fields, arbitrary cutting planes, mixed RK4 /
RKF45, different store types) through one launch per store type and one
captured CUDA graph.

* each job's Q from the batch equals the same job solved alone in a batch of
  one (bit for bit: the same kernels run the same lines);
* each job agrees with the single-job pipeline QMapPlan (same store, same
  settings) on the NaN mask and to 1e-5 in log10 Q;
* replaying the captured graph reproduces the direct run.
"""
import numpy as np
import pytest
import torch

from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu


def _specs(device="cuda"):
    from fastqsl_gb300 import api, synthetic as S
    rng = np.random.default_rng(42)
    shapes = [(48, 48, 48), (64, 56, 40), (40, 40, 32), (56, 48, 48), (44, 52, 36)]
    layouts = ["h4b", "f4", "soa", "h4b", "h8c"]
    specs, stores = [], []
    for k, (shape, layout) in enumerate(zip(shapes, layouts)):
        spec = S.charges_random(100 + k, shape, int(rng.integers(4, 12)))
        B = S.make_field(spec)
        fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout=layout)
        stores.append(fs)
        n0, n1 = int(rng.integers(12, 30)), int(rng.integers(12, 30))
        normal = rng.normal(size=3)
        xs, ys, zs, nrm, stride = S.cutting_plane(shape, normal, n0, n1)
        if k % 2 == 0:
            prm = P.absolute_rkf45(tol=10 ** rng.uniform(-5, -3))
        else:
            prm = P.fixed_rk4(arith=P.ARITH_FAST)
        specs.append(dict(field=fs, xs=torch.from_numpy(xs).to(device), ys=torch.from_numpy(ys).to(device),
                          zs=torch.from_numpy(zs).to(device), n0=n0, n1=n1, nplanes=1, params=prm,
                          s_len=0.25 if k % 2 == 0 else 0.2, stride=stride, cross_dir=tuple(float(c) for c in nrm)))
    return specs, stores


def test_batch_alone_equals_mixed_and_graph(cuda):
    from fastqsl_gb300 import api
    specs, stores = _specs()
    qb = api.QBatch(specs)
    mixed = [q.cpu().numpy() for q in qb.run()]
    torch.cuda.synchronize()
    for k, sp in enumerate(specs):
        alone = api.QBatch([sp]).run()[0].cpu().numpy()
        np.testing.assert_array_equal(alone, mixed[k])
    qb.capture()
    for q in qb.jobs:
        q["Q"].fill_(-7.0)
    replay = [q.cpu().numpy() for q in qb.replay()]
    torch.cuda.synchronize()
    for a, b in zip(replay, mixed):
        np.testing.assert_array_equal(a, b)


def test_batch_matches_single_job_pipeline(cuda):
    from fastqsl_gb300 import api
    specs, stores = _specs()
    Qb = [q.cpu().numpy() for q in api.QBatch(specs).run()]
    for sp, qb in zip(specs, Qb):
        plan = api.QMapPlan(sp["n0"], sp["n1"], 1)
        q1 = plan.run(sp["field"], sp["xs"], sp["ys"], sp["zs"], sp["params"], s_len=sp["s_len"],
                      stride=sp["stride"], cross_dir=sp["cross_dir"]).cpu().numpy()
        assert (np.isnan(q1) == np.isnan(qb)).mean() >= 0.99
        ok = ~np.isnan(q1) & ~np.isnan(qb)
        d = np.abs(np.log10(q1[ok]) - np.log10(qb[ok]))
        assert np.median(d) <= 1e-5, np.median(d)


def test_batch_register_budgets_agree_and_tuner_applies(cuda):
    """The batched kernels compiled for 6-10 resident blocks per SM give the
    same Q maps bit for bit (only the register allocation differs); the
    autotuner's choice is one of them and is what the batch then runs with,
    captured graph included."""
    from fastqsl_gb300 import api, autotune
    specs, stores = _specs()
    qb = api.QBatch(specs)
    ref = [q.cpu().numpy() for q in qb.run()]
    for occ in (6, 7, 9, 10):
        qb.occupancy = occ
        got = [q.cpu().numpy() for q in qb.run()]
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)
    res = autotune.tune_batch(qb, windows=4, window_lines=1024)
    assert res["occupancy"] in autotune.BATCH_OCCUPANCIES and qb.occupancy == res["occupancy"]
    assert set(res["table"]) == {f"occ{o}" for o in autotune.BATCH_OCCUPANCIES}
    qb.capture()
    got = [q.cpu().numpy() for q in qb.replay()]
    torch.cuda.synchronize()
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
