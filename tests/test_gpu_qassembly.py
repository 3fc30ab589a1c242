"""GPU Q assembly through the C ABI.

* Drop-in FastQSL.QCalcPlane / CookPseudoLine / QCalcCut / QMerge on the
  reference's own traced footpoints: bit-identical to the reference's Q
  (golden fixture made by running fastqslpy/FastQSL.py and the notebook
  cells).
* The notebook workflow end to end through the drop-in (kernels + FastQSL).
* The native on-device pipeline (QMapPlan) against the FP64 oracle pipeline:
  median |dlog10 Q| <= 1e-3, 99th percentile <= 1e-2.
"""
import numpy as np
import pytest
import torch

import golden_util as G
from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu


def _d(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def test_qcalc_plane_cook_qcut_bitexact(cuda):
    from fastqsl_gb300.fastqslpy import FastQSL
    g, meta = G.load("qmap_rkf45_bipole4_64.npz")
    shp = tuple(meta["xy_shape"])
    r = lambda k: _d(g["main_" + k].reshape(shp))  # noqa: E731
    stride_step = 1 / meta["interp_ratio"]
    Q = FastQSL.QCalcPlane(r("end_x"), r("end_y"), r("end_z"), r("flag_end"), r("start_x"), r("start_y"),
                           r("start_z"), r("flag_start"), r("B_start_x"), r("B_start_y"), r("B_start_z"),
                           r("B_end_x"), r("B_end_y"), r("B_end_z"), r("B_this_x"), r("B_this_y"), r("B_this_z"),
                           r("B_flag"), stride_step)
    np.testing.assert_array_equal(Q.cpu().numpy(), g["Q"])
    stride_this = np.float32(1.0 / meta["interp_ratio"])
    cook = FastQSL.CookPseudoLine(r("end_x"), r("end_y"), r("end_z"), r("flag_end"), r("start_x"), r("start_y"),
                                  r("start_z"), r("flag_start"), r("B_start_x"), r("B_start_y"), r("B_start_z"),
                                  r("B_end_x"), r("B_end_y"), r("B_end_z"), r("B_this_z"), r("B_flag"), stride_this)
    assert len(cook) == 25
    np.testing.assert_array_equal(cook[0].cpu().numpy(), g["cut_inp_x"])
    np.testing.assert_array_equal(cook[1].cpu().numpy(), g["cut_inp_y"])
    np.testing.assert_array_equal(cook[2].cpu().numpy(), g["cut_inp_z"])
    np.testing.assert_array_equal(cook[23].cpu().numpy(), g["Bz0_start"])
    np.testing.assert_array_equal(cook[24].cpu().numpy(), g["Bz0_end"])
    assert int(cook[21].cpu().to(torch.int64).item()) == g["cut_inp_x"].size
    c = lambda k: _d(g["cut_" + k])  # noqa: E731
    Qc = FastQSL.QCalcCut(c("start_x"), c("start_y"), c("start_z"), c("flag_start"), c("end_x"), c("end_y"),
                          c("end_z"), c("flag_end"), _d(g["Bz0_start"]), _d(g["Bz0_end"]), stride_this)
    np.testing.assert_array_equal(Qc.cpu().numpy(), g["Qcut"])
    _, Qf = FastQSL.QMerge(Q, Qc, r("B_flag"))
    np.testing.assert_array_equal(Qf.cpu().numpy(), g["Q_final"])


def test_cook_empty_and_all_flagged(cuda):
    from fastqsl_gb300.fastqslpy import FastQSL
    n0, n1 = 7, 9
    z = torch.zeros((n0, n1), dtype=torch.float32, device="cuda")
    fl = torch.full((n0, n1), 5, dtype=torch.int32, device="cuda")
    none = torch.zeros((n0, n1), dtype=torch.int32, device="cuda")
    out = FastQSL.CookPseudoLine(z, z, z, fl, z + 3, z + 4, z, fl, z, z, z + 1, z, z, z + 2, z, none, 0.5)
    assert out[0].numel() == 0 and out[23].numel() == 0
    allf = torch.ones((n0, n1), dtype=torch.int32, device="cuda")
    out = FastQSL.CookPseudoLine(z, z, z, fl, z + 3, z + 4, z, fl, z, z, z + 1, z, z, z + 2, z, allf, 0.5)
    assert out[0].numel() == 4 * n0 * n1
    xs = out[0].cpu().numpy().reshape(-1, 4)
    ys = out[1].cpu().numpy().reshape(-1, 4)
    np.testing.assert_array_equal(xs[:, 0], 3.5)
    np.testing.assert_array_equal(xs[:, 2], 2.5)
    np.testing.assert_array_equal(ys[:, 1], 4.5)
    np.testing.assert_array_equal(ys[:, 3], 3.5)


def test_notebook_workflow_through_dropin(cuda):
    """demo/Q_RKF45CuPy.ipynb cells 6-11 run against the drop-in: the final Q
    map matches the reference's."""
    from fastqsl_gb300.fastqslpy import FastQSL, kernels
    from test_gpu_trace import _field_dev
    g, meta = G.load("qmap_rkf45_bipole4_64.npz")
    Bx, By, Bz = G.field_for(meta)
    bx, by, bz = _field_dev(Bx, By, Bz)
    shp = tuple(meta["xy_shape"])
    n = shp[0] * shp[1]
    TraceAllBline = kernels.compileTraceBlineAdaptive()
    BshapeN = torch.tensor(list(Bx.shape), dtype=torch.int32, device="cuda")
    dummy = torch.zeros((1, 1), dtype=torch.float32, device="cuda")
    flag_twist = torch.tensor([False], device="cuda")

    def alloc(m):
        f = [torch.zeros(m, dtype=torch.float32, device="cuda") for _ in range(15)]
        i = [torch.zeros(m, dtype=torch.int32, device="cuda") for _ in range(3)]
        return f, i

    (x_start, y_start, z_start, x_end, y_end, z_end, Bx_start, By_start, Bz_start, Bx_end, By_end, Bz_end,
     Bx_inp, By_inp, Bz_inp), (B_flag, flag_start, flag_end) = alloc(n)
    line_len = torch.zeros(n, dtype=torch.float64, device="cuda")
    N = torch.tensor([n], dtype=torch.int64, device="cuda")
    s_len = torch.tensor([meta["s_len"]], dtype=torch.float32, device="cuda")
    tol_coef = torch.tensor([meta["tol_coef"]], dtype=torch.float32, device="cuda")
    inp_norm = torch.tensor([0, 0, 1.0], dtype=torch.float32, device="cuda")
    x_inp, y_inp, z_inp = _d(g["inp_x"]), _d(g["inp_y"]), _d(g["inp_z"])
    TraceAllBline((128, 1, 1), (28, 1),
                  (bx, by, bz, BshapeN, dummy, dummy, dummy, dummy, flag_twist, x_inp, y_inp, z_inp, inp_norm,
                   x_start, y_start, z_start, flag_start, x_end, y_end, z_end, flag_end, Bx_inp, By_inp, Bz_inp,
                   B_flag, Bx_start, By_start, Bz_start, Bx_end, By_end, Bz_end, s_len, N, line_len,
                   tol_coef * 0.5))
    arrs = FastQSL.ResReshape(shp, x_end, y_end, z_end, flag_end, x_start, y_start, z_start, flag_start,
                              Bx_start, By_start, Bz_start, Bx_end, By_end, Bz_end, Bx_inp, By_inp, Bz_inp, B_flag)
    stride_step = 1 / meta["interp_ratio"]
    Q = FastQSL.QCalcPlane(*arrs, stride_step)
    stride_this = np.float32(1.0 / meta["interp_ratio"])
    cook = FastQSL.CookPseudoLine(*arrs[:14], arrs[16], arrs[17], stride_this)
    (cut_inp_x, cut_inp_y, cut_inp_z, cut_start_x, cut_start_y, cut_start_z, flag_cut_start, cut_end_x, cut_end_y,
     cut_end_z, flag_cut_end, Bx_inp_cut, By_inp_cut, Bz_inp_cut, B_flag_cut, Bx_start_cut, By_start_cut,
     Bz_start_cut, Bx_end_cut, By_end_cut, Bz_end_cut, N_cut, line_len_cut, Bz0_start, Bz0_end) = cook
    TraceAllBline((128, 1, 1), (28, 1),
                  (bx, by, bz, BshapeN, dummy, dummy, dummy, dummy, flag_twist, cut_inp_x, cut_inp_y, cut_inp_z,
                   inp_norm, cut_start_x, cut_start_y, cut_start_z, flag_cut_start, cut_end_x, cut_end_y, cut_end_z,
                   flag_cut_end, Bx_inp_cut, By_inp_cut, Bz_inp_cut, B_flag_cut, Bx_start_cut, By_start_cut,
                   Bz_start_cut, Bx_end_cut, By_end_cut, Bz_end_cut, s_len, N_cut, line_len_cut, tol_coef * .1))
    Qcut = FastQSL.QCalcCut(cut_start_x, cut_start_y, cut_start_z, flag_cut_start, cut_end_x, cut_end_y, cut_end_z,
                            flag_cut_end, Bz0_start, Bz0_end, stride_this)
    _, Q_final = FastQSL.QMerge(Q, Qcut, arrs[17])
    got = Q_final.cpu().numpy()
    ref = g["Q_final"]
    flags_same = ((flag_start.cpu().numpy() == g["main_flag_start"]) &
                  (flag_end.cpu().numpy() == g["main_flag_end"])).mean()
    assert flags_same >= 0.999, flags_same
    # one differing flag changes the NaN mask of at most 5 pixels
    nan_same = (np.isnan(got) == np.isnan(ref)).mean()
    assert nan_same >= 1.0 - 5.0 * (1.0 - flags_same) - 1e-9, (nan_same, flags_same)
    ok = ~np.isnan(got) & ~np.isnan(ref)
    d = np.abs(np.log10(got[ok]) - np.log10(ref[ok]))
    assert np.median(d) <= 1e-6 and np.quantile(d, 0.99) <= 1e-2, (np.median(d), np.quantile(d, 0.99))


@pytest.mark.parametrize("layout,arith", [("f4", P.ARITH_FAST), ("soa", P.ARITH_FAST), ("h4b", P.ARITH_FAST),
                                          ("h8c", P.ARITH_FAST), ("h4b", P.ARITH_FAST_W16)])
def test_qmap_pipeline_vs_fp64_oracle(cuda, oracle_port, layout, arith):
    from fastqsl_gb300 import api, synthetic as S
    from oracle import qassembly as QA
    spec = S.charges_random(21, (80, 72, 48), 6)
    Bx, By, Bz = S.make_field(spec)
    n0, n1 = 40, 48
    zs = [0.0, 6.0, 13.5]
    stride = 1.5
    xs, ys, zz = api.plane_seed_grid(4.0, 4.0 + stride * (n1 - 1), n1, 4.0, 4.0 + stride * (n0 - 1), n0, zs)
    prm = P.absolute_rkf45(arith=arith)
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout=layout)
    plan = api.QMapPlan(n0, n1, len(zs))
    Q = plan.run(fs, xs, ys, zz, prm, s_len=0.25, stride=stride).cpu().numpy()
    prm64 = P.absolute_rkf45(arith=P.ARITH_EXACT)
    tr = lambda a, b, c: oracle_port.trace_all("port64", Bx, By, Bz, a, b, c, s_len=0.25, params=prm64)  # noqa
    Qref = QA.qmap_pipeline(tr, xs.cpu().numpy(), ys.cpu().numpy(), zz.cpu().numpy(), len(zs), n0, n1, stride)
    nan_same = np.isnan(Q) == np.isnan(Qref)
    assert nan_same.mean() >= 0.99
    ok = ~np.isnan(Q) & ~np.isnan(Qref)
    d = np.abs(np.log10(Q[ok]) - np.log10(Qref[ok]))
    # every form with FP32 interpolation meets median <= 1e-3 and 99th
    # percentile <= 1e-2; the opt-in fp16-x-weight sampler's tail on this
    # steep small field is within 5e-2 (its stated bar)
    p99_bar = 5e-2 if arith == P.ARITH_FAST_W16 else 1e-2
    assert np.median(d) <= 1e-3 and np.quantile(d, 0.99) <= p99_bar, (np.median(d), np.quantile(d, 0.99))


@pytest.mark.parametrize("layout", ["h4b", "soa"])
def test_field_uploader_pipeline(cuda, layout):
    """Fields uploaded from pinned host memory through FieldUploader, the next
    field's copy queued before the current field's Q map: every Q map equals
    the one from a store built directly from that field, bit for bit."""
    from fastqsl_gb300 import api, synthetic as S
    shape = (56, 48, 40)
    fields = [S.make_field(S.charges_random(30 + k, shape, 4 + k)) for k in range(3)]
    n0, n1 = 24, 28
    xs, ys, zz = api.plane_seed_grid(3.0, 3.0 + 1.5 * (n1 - 1), n1, 3.0, 3.0 + 1.5 * (n0 - 1), n0, [0.0, 5.0])
    prm = P.absolute_rkf45()
    plan = api.QMapPlan(n0, n1, 2)
    ref = []
    for B in fields:
        fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout=layout)
        ref.append(plan.run(fs, xs, ys, zz, prm, s_len=0.25, stride=1.5).cpu().numpy())
        fs.close()
    hosts = [[torch.from_numpy(np.ascontiguousarray(b.transpose(2, 1, 0))).pin_memory() for b in B] for B in fields]
    up = api.FieldUploader(shape)
    store = api.FieldStore(*[torch.zeros(shape[::-1], device="cuda").permute(2, 1, 0) for _ in range(3)],
                           layout=layout)
    st = torch.cuda.current_stream()
    outs = []
    slot = up.upload(*hosts[0])
    for k in range(len(fields)):
        up.pack(store, slot, st)
        if k + 1 < len(fields):
            slot = up.upload(*hosts[k + 1])
        q = plan.run(store, xs, ys, zz, prm, s_len=0.25, stride=1.5)
        h = torch.empty(q.shape, dtype=q.dtype).pin_memory()
        h.copy_(q, non_blocking=True)
        outs.append(h)
    torch.cuda.synchronize()
    for a, b in zip(outs, ref):
        a = a.numpy()
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        np.testing.assert_array_equal(a[~np.isnan(a)], b[~np.isnan(b)])
    with pytest.raises(ValueError):
        up.upload(*[h[:-1] for h in hosts[0]])


@pytest.mark.parametrize("layout", ["h4b", "f4"])
def test_qseries_pipeline(cuda, layout):
    """A series of host fields through api.QSeries (two stores, two plans:
    uploads, packs and Q copies to the host overlapping the neighbouring
    fields' traces): every field's Q equals the Q of a plan run on a store
    built directly from that field, bit for bit, with four fields
    alternating over the two stores."""
    from fastqsl_gb300 import api, synthetic as S
    shape = (56, 48, 40)
    fields = [S.make_field(S.charges_random(40 + k, shape, 4 + k)) for k in range(4)]
    n0, n1 = 24, 28
    xs, ys, zz = api.plane_seed_grid(3.0, 3.0 + 1.5 * (n1 - 1), n1, 3.0, 3.0 + 1.5 * (n0 - 1), n0, [0.0, 5.0])
    prm = P.absolute_rkf45()
    plan = api.QMapPlan(n0, n1, 2)
    ref = []
    for B in fields:
        fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout=layout)
        ref.append(plan.run(fs, xs, ys, zz, prm, s_len=0.25, stride=1.5).cpu().numpy())
        fs.close()
    hosts = [[torch.from_numpy(np.ascontiguousarray(b.transpose(2, 1, 0))).pin_memory() for b in B] for B in fields]
    series = api.QSeries(shape, n0, n1, 2, layout=layout)
    outs = [torch.empty((2, n0 - 2, n1 - 2), dtype=torch.float64).pin_memory() for _ in fields]
    for h, q in zip(hosts, outs):
        series.push(*h, xs, ys, zz, prm, q, s_len=0.25, stride=1.5)
    series.wait()
    torch.cuda.synchronize()
    for a, b in zip(outs, ref):
        a = a.numpy()
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        np.testing.assert_array_equal(a[~np.isnan(a)], b[~np.isnan(b)])
    series.close()
