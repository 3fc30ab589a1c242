"""The native Q-map batch (qsl_qmap_batch_*) against the Python-built batch
of the same jobs (QBatch over qsl_plane_seeds / qsl_tile_order seeds): the
same trace kernels, and the Q assembly, compaction, pseudo Q and merge as
one launch each over a job table with the per-job kernels' arithmetic, so
every Q map must be equal bit for bit, whole and run as windows of the main
trace, for planes of any orientation, several fields, tolerances and
sub-boxes of stacked planes."""
import numpy as np
import pytest
import torch

from fastqsl_gb300 import api, params as P

pytestmark = pytest.mark.gpu


def _same(a, b):
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert a.shape == b.shape
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(a)
    np.testing.assert_array_equal(a[ok], b[ok])


@pytest.fixture(scope="module")
def fields(cuda):
    from fastqsl_gb300 import serving
    fs = serving.make_fields(n_fields=2, shape=(48, 44, 40), seed=3)
    yield fs
    for f in fs.values():
        f.close()


def _jobs(fields):
    from fastqsl_gb300 import serving
    geo = [("f0", (24.0, 22.0, 6.0), (0.0, 0.0, 1.0), 1.0, 17, 23, 1, 1e-4),
           ("f1", (20.0, 21.0, 14.0), (0.3, -0.2, 0.93), 0.7, 25, 19, 3, 1e-3),
           ("f0", (26.0, 20.0, 18.0), (1.0, 0.0, 0.0), 0.5, 9, 40, 2, 1e-5),
           ("f1", (22.0, 22.0, 9.0), (0.0, 1.0, 0.0), 1.3, 3, 3, 1, 1e-4)]
    jobs = []
    for name, c, nrm, sp, n0, n1, npl, tol in geo:
        n, u, v = serving.plane_axes(nrm)
        jobs.append(dict(field=fields[name], params=P.absolute_rkf45(tol=tol), center=c, normal=n, u=u, v=v,
                         spacing=sp, n0=n0, n1=n1, nplanes=npl, s_len=0.25, tol_coef=1.0))
    return jobs


def _qbatch(jobs, tile):
    specs = []
    for j in jobs:
        xs, ys, zs = api.plane_seeds(j["center"], j["normal"], j["u"], j["v"], j["spacing"], j["n0"], j["n1"],
                                     j["nplanes"])
        specs.append(dict(field=j["field"], xs=xs, ys=ys, zs=zs, n0=j["n0"], n1=j["n1"], nplanes=j["nplanes"],
                          params=j["params"], s_len=j["s_len"], stride=j["spacing"], cross_dir=j["normal"]))
    return api.QBatch(specs, tile=tile)


@pytest.mark.parametrize("tile", [(8, 8), None])
def test_native_batch_equals_python_batch(fields, tile):
    jobs = _jobs(fields)
    ref = [q.clone() for q in _qbatch(jobs, tile).run()]
    nb = api.PlaneQBatch(jobs, tile=tile)
    got = nb.run()
    torch.cuda.synchronize()
    assert len(got) == len(jobs)
    for a, b in zip(ref, got):
        _same(a, b)
    assert sum(int(torch.isfinite(q).sum()) for q in got) > 0.9 * sum(q.numel() for q in got)
    nb.close()


def test_native_batch_many_jobs(fields):
    """Eleven jobs, several with more than one compaction tile (1024 pixels)
    and Q grid block per plane, so that the batched Q-assembly launches map
    blocks to jobs across uneven block ranges."""
    from fastqsl_gb300 import serving
    geo = [((24.0, 22.0, 8.0), (0.0, 0.0, 1.0), 0.3, 64, 50, 1), ((24.0, 22.0, 12.0), (0.2, 0.1, 0.97), 0.25, 41, 37, 2),
           ((23.0, 21.0, 15.0), (1.0, 0.0, 0.0), 0.4, 33, 61, 1), ((22.0, 22.0, 9.0), (0.0, 1.0, 0.0), 0.5, 5, 4, 1),
           ((25.0, 20.0, 20.0), (0.0, 0.0, 1.0), 0.6, 3, 3, 2), ((24.0, 24.0, 6.0), (0.5, -0.5, 0.7), 0.2, 70, 70, 1),
           ((21.0, 23.0, 10.0), (0.0, 0.0, 1.0), 0.35, 17, 90, 3), ((20.0, 22.0, 18.0), (0.0, 1.0, 0.0), 0.3, 48, 48, 1),
           ((26.0, 21.0, 7.0), (0.0, 0.0, 1.0), 0.8, 9, 11, 4), ((24.0, 22.0, 14.0), (1.0, 0.0, 0.0), 0.25, 65, 33, 1),
           ((22.0, 20.0, 11.0), (0.3, 0.3, 0.9), 0.45, 29, 31, 2)]
    jobs = []
    for k, (c, nrm, sp, n0, n1, npl) in enumerate(geo):
        n, u, v = serving.plane_axes(nrm)
        jobs.append(dict(field=fields["f%d" % (k % 2)], params=P.absolute_rkf45(tol=(1e-4, 1e-3)[k % 2]), center=c,
                         normal=n, u=u, v=v, spacing=sp, n0=n0, n1=n1, nplanes=npl, s_len=0.25, tol_coef=1.0))
    ref = [q.clone() for q in _qbatch(jobs, (8, 8)).run()]
    nb = api.PlaneQBatch(jobs, tile=(8, 8))
    got = nb.run()
    torch.cuda.synchronize()
    for a, b in zip(ref, got):
        _same(a, b)
    assert sum(int(torch.isfinite(q).sum()) for q in got) > 0.8 * sum(q.numel() for q in got)
    nb.close()


def test_native_batch_windows(fields):
    jobs = _jobs(fields)
    whole = [q.clone() for q in api.PlaneQBatch(jobs).run()]
    nb = api.PlaneQBatch(jobs, blocks_per_sm=2)
    lines = nb.main_lines
    assert lines > 0 and lines % 32 == 0
    step = 96
    for lo in range(0, lines, step):
        nb.run_main(lo=lo, hi=min(lines, lo + step))
    got = nb.run_post()
    torch.cuda.synchronize()
    for a, b in zip(whole, got):
        _same(a, b)


def test_native_batch_rejects_bad_jobs(fields):
    from fastqsl_gb300 import _lib
    jobs = _jobs(fields)
    jobs[1]["n0"] = 2
    with pytest.raises(_lib.QslError):
        api.PlaneQBatch(jobs)
    jobs = _jobs(fields)
    jobs[0]["params"] = P.absolute_rkf45(arith=P.ARITH_EXACT)
    with pytest.raises(_lib.QslError):
        api.PlaneQBatch(jobs)
