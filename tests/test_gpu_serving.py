"""The continuous-batching server: results identical alone and in the mix,
HBM-budget admission, latency statistics."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _server(budget=8 << 30, streams=2, max_batch=8):
    from fastqsl_gb300 import serving
    fields = serving.make_fields(n_fields=3, shape=(48, 44, 40), seed=3)
    return serving.QServer(fields, hbm_budget=budget, streams=streams, max_batch=max_batch), (48, 44, 40)


def _same(a, b):
    assert a.shape == b.shape
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(a)
    np.testing.assert_array_equal(a[ok], b[ok])


def test_alone_equals_mixed(cuda):
    from fastqsl_gb300 import serving
    srv, shape = _server()
    reqs = serving.make_requests(shape, sorted(srv.fields), 14, None, seed=5, seeds_range=(200, 3000))
    alone = {r.rid: serving.solve_alone(srv, r) for r in reqs}
    done = srv.run_stream(reqs)
    assert len(done) == len(reqs) and srv.idle()
    assert srv.batches >= 2 + len(reqs)  # the burst ran in batches of up to 8
    for r in done:
        _same(r.result, alone[r.rid][1])
        assert r.result.shape == (r.nplanes, r.n0 - 2, r.n1 - 2)
    st = serving.latency_stats(done, {k: v[0] for k, v in alone.items()})
    assert st["p99_s"] >= st["p50_s"] > 0 and st["qpixels_per_s"] > 0


def test_budget_admission_and_poisson_stream(cuda):
    from fastqsl_gb300 import serving
    reqs0 = serving.make_requests((48, 44, 40), ["f0", "f1", "f2"], 10, 400.0, seed=9, seeds_range=(500, 2500))
    biggest = max(serving.request_bytes(r) for r in reqs0)
    srv, shape = _server(budget=biggest + 1)  # one request in flight at a time
    alone = {r.rid: serving.solve_alone(srv, r)[1] for r in reqs0}
    done = srv.run_stream(reqs0)
    assert srv.used == 0 and len(done) == 10
    assert srv.batches >= 12  # the stream could not be admitted as one batch
    for r in done:
        _same(r.result, alone[r.rid])
        assert r.t_submit <= r.t_admit <= r.t_done
    big = serving.QRequest(rid=99, field="f0", n0=400, n1=400)
    with pytest.raises(MemoryError):
        srv.submit(big)


def test_windowed_bulk_equals_whole(cuda):
    """Larger classes' main traces run as windows of a few lines (forced
    small here, with a window limit of 1 while small batches fly): every
    result equals the one-launch server's bit for bit."""
    from fastqsl_gb300 import serving
    fields = serving.make_fields(n_fields=3, shape=(48, 44, 40), seed=3)
    classes = ((600, 4, 2), (1500, 4, 2), (float("inf"), 2, 2))
    whole = serving.QServer(fields, streams=2, classes=classes, chunk_lines=0)
    win = serving.QServer(fields, streams=2, classes=classes, chunk_lines=96, max_chunks=2,
                          chunks_when_interactive=1)
    assert win.chunk_lines == 96
    reqs = serving.make_requests((48, 44, 40), sorted(fields), 12, 300.0, seed=11, seeds_range=(200, 4000))
    assert len({next(c for c, (ub, _, _) in enumerate(classes) if r.seeds <= ub) for r in reqs}) == 3
    ref = {r.rid: r.result for r in whole.run_stream(reqs)}
    reqs2 = serving.make_requests((48, 44, 40), sorted(fields), 12, 300.0, seed=11, seeds_range=(200, 4000))
    done = win.run_stream(reqs2)
    assert len(done) == 12 and win.idle() and win.used == 0
    for r in done:
        _same(r.result, ref[r.rid])
