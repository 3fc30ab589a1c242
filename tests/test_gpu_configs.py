"""The smaller benchmark configurations at their full sizes.

* 64^3 potential field of 4 charges, 128x128 seeds on z = 0, RK4 with the
  reference's fixed step 0.1 and 20000-step limit: the drop-in RK4 entry
  (exact arithmetic) against the oracle restatement of the reference's
  TraceBline.cu, which is bit-identical to the reference on its golden
  fixtures.
* 256x256x128 bipole + twisted flux tube, a 512x256 seed plane at 2x
  refinement (spacing 0.5) on z = 0, RKF45 tol 1e-4, h in [1e-3, 1]: the
  native Q pipeline on fp16 bricks against the FP64 oracle on a seeded sample
  of pixels (each recomputed from its 3x3 seed stencil and, where flagged,
  its pseudo-lines), plus properties that hold at any size.
"""
import numpy as np
import pytest
import torch

from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu


def test_config1_rk4_dropin_full_size(cuda, oracle_port):
    from test_gpu_trace import run_dropin
    from fastqsl_gb300 import synthetic as S
    Bx, By, Bz = S.make_field(S.bipole4_64(0))
    g = np.linspace(0.0, 63.0, 128, dtype=np.float32)
    X, Y = np.meshgrid(g, g)
    xs, ys = X.ravel().astype(np.float32), Y.ravel().astype(np.float32)
    zs = np.zeros_like(xs)
    got = run_dropin("rk4", Bx, By, Bz, xs, ys, zs, 0.1, 1.0)
    ref = oracle_port.trace_all("port32", Bx, By, Bz, xs, ys, zs, s_len=0.1, tol_coef=1.0,
                                params=P.reference_rk4())
    assert (got["flag_start"] == ref["flag_start"]).all() and (got["flag_end"] == ref["flag_end"]).all()
    live = (ref["flag_start"] != 0) & (ref["flag_end"] != 0)
    assert live.mean() > 0.5
    for k in ("start_x", "start_y", "start_z", "end_x", "end_y", "end_z"):
        assert (got[k][live] == ref[k][live]).mean() >= 0.999, k
    np.testing.assert_array_equal(got["B_flag"], ref["B_flag"])


def test_config2_qmap_full_size(cuda, oracle_port):
    from fastqsl_gb300 import api, synthetic as S
    from oracle import qassembly as QA
    spec = S.bipole_tube_256()
    Bd = S.make_field(spec, device="cuda", as_numpy=False)
    n1, n0 = 512, 256                      # 512 seeds along x, 256 along y, spacing 0.5
    x0, y0 = 0.0, 64.0
    xs, ys, zz = api.plane_seed_grid(x0, x0 + 0.5 * (n1 - 1), n1, y0, y0 + 0.5 * (n0 - 1), n0, [1e-4], device="cuda")
    prm = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=P.ARITH_FAST)
    store = api.FieldStore(*Bd, layout="h4b")
    plan = api.QMapPlan(n0, n1, 1)
    Q = plan.run(store, xs, ys, zz, prm, s_len=0.25, stride=0.5)[0].cpu().numpy()
    torch.cuda.synchronize()
    assert Q.shape == (n0 - 2, n1 - 2)
    fin = np.isfinite(Q)
    assert fin.mean() > 0.9 and (Q[fin] >= 1.0).all()
    # a pixel next to a change of exit face stays NaN (pseudo-lines replace
    # only flagged pixels whose stencil does not jump)
    fs = plan.main["flag_start"].view(n0, n1).cpu().numpy()
    fe = plan.main["flag_end"].view(n0, n1).cpu().numpy()
    c = (slice(1, -1), slice(1, -1))
    jump = np.zeros((n0 - 2, n1 - 2), bool)
    for F in (fs, fe):
        for sh in ((slice(2, None), slice(1, -1)), (slice(0, -2), slice(1, -1)), (slice(1, -1), slice(2, None)),
                   (slice(1, -1), slice(0, -2))):
            jump |= F[sh] != F[c]
    assert not (fin & jump).any()
    # the FP64 oracle on 300 seeded interior pixels
    rng = np.random.default_rng(2024)
    ci = rng.integers(0, n0 - 2, 300)
    cj = rng.integers(0, n1 - 2, 300)
    B = [np.asfortranarray(b.cpu().numpy()) for b in Bd]
    sx, sy, sz = [], [], []
    for i, j in zip(ci, cj):
        for a in range(3):
            for b in range(3):
                sx.append(x0 + 0.5 * (j + b))
                sy.append(y0 + 0.5 * (i + a))
                sz.append(1e-4)
    sx, sy, sz = (np.array(v, np.float32) for v in (sx, sy, sz))
    prm64 = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=P.ARITH_EXACT)
    tr = lambda a, b, cc: oracle_port.trace_all("port64", B[0], B[1], B[2], a, b, cc, s_len=0.25,  # noqa: E731
                                                params=prm64)
    Qr = QA.qmap_pipeline(tr, sx, sy, sz, 300, 3, 3, 0.5)[:, 0, 0]
    Qg = Q[ci, cj]
    assert (np.isnan(Qr) == np.isnan(Qg)).mean() >= 0.98
    both = ~np.isnan(Qr) & ~np.isnan(Qg)
    d = np.abs(np.log10(Qg[both]) - np.log10(Qr[both]))
    assert np.median(d) <= 1e-3 and np.quantile(d, 0.99) <= 1e-2, (np.median(d), np.quantile(d, 0.99))
