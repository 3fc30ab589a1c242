"""GPU tracer parity through the C ABI.

* The drop-in entry (fastqslpy.kernels, exact arithmetic) against the
  reference's own outputs (golden fixtures): RK4 bit-exact; RKF45 bit-exact
  against the oracle built with the same correctly rounded power function,
  and within the bars (>= 99.9 % identical flags, footpoints within 1e-3
  cell) against the reference's host build, whose powf rounds differently
  in ~6e-4 of calls.
* The fast FP32 kernels (SoA, interleaved float4, fp16 bricks) against the
  oracle at the benchmark settings: flags identical for >= 99.8 %,
  footpoints within 1e-3 cell for >= 99 % (2e-2 cell with fp16 storage; on
  a field the fp16 stores hold exactly, 1e-3 cell as for float32).
"""
import numpy as np
import pytest
import torch

import golden_util as G
from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu


def _dev(a, dtype=None):
    t = torch.as_tensor(np.asarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def _field_dev(Bx, By, Bz):
    from fastqsl_gb300.api import as_xfast
    return [as_xfast(torch.from_numpy(np.asfortranarray(b))) for b in (Bx, By, Bz)]


def run_dropin(kind, Bx, By, Bz, xs, ys, zs, s_len, tol_coef, curB=None, cross=(0, 0, 1), arith="exact"):
    from fastqsl_gb300.fastqslpy import kernels
    k = kernels.compileTraceBlineAdaptive(arith) if kind == "rkf45" else kernels.compileTraceBlineRK4(arith)
    bx, by, bz = _field_dev(Bx, By, Bz)
    shape = torch.tensor(list(Bx.shape), dtype=torch.int32, device="cuda")
    n = len(xs)
    f32 = lambda: torch.zeros(n, dtype=torch.float32, device="cuda")  # noqa: E731
    i32 = lambda: torch.zeros(n, dtype=torch.int32, device="cuda")  # noqa: E731
    o = {k2: f32() for k2 in ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z", "B_this_x", "B_this_y",
                              "B_this_z", "B_start_x", "B_start_y", "B_start_z", "B_end_x", "B_end_y", "B_end_z"]}
    o.update({k2: i32() for k2 in ["flag_start", "flag_end", "B_flag"]})
    o["LineLen"] = torch.zeros(n, dtype=torch.float64, device="cuda")
    o["twist"] = torch.zeros(n, dtype=torch.float64, device="cuda")
    dummy = torch.zeros((1, 1), dtype=torch.float32, device="cuda")
    if curB is not None:
        cx, cy, cz = _field_dev(*curB)
        flag = torch.tensor([True], device="cuda")
    else:
        cx = cy = cz = dummy
        flag = torch.tensor([False], device="cuda")
    args = [bx, by, bz, shape, cx, cy, cz, o["twist"], flag,
            _dev(xs), _dev(ys), _dev(zs), torch.tensor(cross, dtype=torch.float32, device="cuda"),
            o["start_x"], o["start_y"], o["start_z"], o["flag_start"],
            o["end_x"], o["end_y"], o["end_z"], o["flag_end"],
            o["B_this_x"], o["B_this_y"], o["B_this_z"], o["B_flag"],
            o["B_start_x"], o["B_start_y"], o["B_start_z"],
            o["B_end_x"], o["B_end_y"], o["B_end_z"],
            torch.tensor([s_len], dtype=torch.float32, device="cuda"),
            torch.tensor([n], dtype=torch.int64, device="cuda"), o["LineLen"]]
    if kind == "rkf45":
        args.append(torch.tensor([tol_coef], dtype=torch.float32, device="cuda"))
    else:
        args.append(torch.tensor([tol_coef], dtype=torch.float32, device="cuda"))  # ignored, as in the notebooks
    k((128, 1, 1), (28, 1), tuple(args))
    torch.cuda.synchronize()
    return {k2: v.cpu().numpy() for k2, v in o.items()}


def foot_dist(a, b):
    return np.sqrt((a["end_x"] - b["end_x"]) ** 2 + (a["end_y"] - b["end_y"]) ** 2 + (a["end_z"] - b["end_z"]) ** 2), \
        np.sqrt((a["start_x"] - b["start_x"]) ** 2 + (a["start_y"] - b["start_y"]) ** 2 +
                (a["start_z"] - b["start_z"]) ** 2)


def check_parity(got, ref, flag_frac=0.999, foot_frac=0.999, tol=1e-3, report=None):
    fs = got["flag_start"] == ref["flag_start"]
    fe = got["flag_end"] == ref["flag_end"]
    both = fs & fe
    de, ds = foot_dist(got, ref)
    live = (ref["flag_start"] != 0) & (ref["flag_end"] != 0)
    close = (de <= tol) & (ds <= tol)
    stats = dict(flags=float(both.mean()), foot=float(close[live].mean()) if live.any() else 1.0,
                 bitexact=float((got["end_x"] == ref["end_x"]).mean()))
    if report is not None:
        report.update(stats)
    assert stats["flags"] >= flag_frac, stats
    assert stats["foot"] >= foot_frac, stats
    return stats


@pytest.mark.parametrize("name", sorted(G.TRACE_CASES))
def test_dropin_exact_matches_reference(cuda, name):
    g, meta = G.load(name)
    kind, twist = G.TRACE_CASES[name]
    Bx, By, Bz = G.field_for(meta)
    cur = G.twist_current(Bx, By, Bz) if twist else None
    got = run_dropin(kind, Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], meta["s_len"], meta["tol_coef"], cur)
    # RK4 is bit-exact to the reference's host build; RKF45's step controller
    # calls a power function whose library rounding differs in ~6e-4 of calls
    # (host powf vs the correctly rounded one used here), which moves some
    # footpoints by the truncation error of the reference's loose tolerance.
    st = check_parity(got, g, foot_frac=0.999 if kind == "rk4" else 0.995)
    if kind == "rk4":
        assert st["bitexact"] > 0.999, st
    # bit-exact against the oracle built with the same (correctly rounded) power
    import oracle
    prm = P.reference_rk4() if kind == "rk4" else P.reference_rkf45()
    cr = oracle.trace_all("port32cr", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], s_len=meta["s_len"],
                          tol_coef=meta["tol_coef"], params=prm, curB=cur)
    live = (cr["flag_start"] != 0) & (cr["flag_end"] != 0)
    for k in ["end_x", "end_y", "end_z", "start_x", "start_y", "start_z"]:
        assert (got[k][live] == cr[k][live]).mean() >= 0.999, k
    assert (got["flag_end"] == cr["flag_end"]).all() and (got["flag_start"] == cr["flag_start"]).all()
    np.testing.assert_array_equal(got["B_this_x"], g["B_this_x"])
    np.testing.assert_array_equal(got["B_flag"], g["B_flag"])
    if twist:  # the current density is sampled on the traced field's grid
        close = np.isclose(got["twist"], cr["twist"], rtol=1e-5, atol=1e-9)
        assert close[live].mean() >= 0.99, close[live].mean()
    same = (got["flag_end"] == g["flag_end"]) & (got["flag_start"] == g["flag_start"])
    rel = np.abs(got["LineLen"] - g["LineLen"]) / np.maximum(g["LineLen"], 1e-6)
    assert np.median(rel[same]) < 1e-6


def test_dropin_fast_arith_rk4_matches_reference(cuda):
    """The TraceBline.cu (RK4) path in fast arithmetic against the reference:
    identical exit faces; footpoints within 1e-3 cell except on the few lines
    next to separatrices, where 3840 fused-multiply-add roundings (and the
    Kahan-compensated position sum, which the reference does not have) move
    them further."""
    g, meta = G.load("trace_rk4_bipole4_64.npz")
    Bx, By, Bz = G.field_for(meta)
    got = run_dropin("rk4", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], meta["s_len"], meta["tol_coef"],
                     arith="fast")
    check_parity(got, g, flag_frac=0.999, foot_frac=0.995)


def test_dropin_fast_arith_rkf45_reference_settings(cuda):
    """RKF45 in fast arithmetic at the reference's loose tolerance
    (1e-3*|b.n|^1.5, steps up to 100 cells): accept/reject decisions sit on
    knife edges, so footpoints move by the truncation error; the exit faces
    still agree.  (Footpoint parity of the fast kernels is checked at the
    benchmark tolerance in test_native_layouts_match_oracle.)"""
    g, meta = G.load("trace_rkf45_bipole4_64.npz")
    Bx, By, Bz = G.field_for(meta)
    got = run_dropin("rkf45", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], meta["s_len"], meta["tol_coef"],
                     arith="fast")
    check_parity(got, g, flag_frac=0.99, foot_frac=0.0)


@pytest.mark.parametrize("layout,sched", [("soa", "static"), ("soa", "queue"), ("f4", "queue"), ("h4b", "queue"),
                                          ("h8c", "static"), ("h8c", "queue")])
def test_native_layouts_match_oracle(cuda, oracle_port, layout, sched):
    """Benchmark settings (RKF45, absolute tol 1e-4, h in [1e-3, 1]) on a
    256x256x128-type field cut down to 96x96x64."""
    from fastqsl_gb300 import api, synthetic as S
    spec = S.charges_random(3, (96, 96, 64), 8)
    Bx, By, Bz = S.make_field(spec)
    xs, ys, zs, shp = S.plane_seeds((2, 93), (2, 93), 72, 72, 0.5)
    prm = P.absolute_rkf45(arith=P.ARITH_FAST)
    ref = oracle_port.trace_all("port32", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0,
                                params=P.absolute_rkf45(arith=P.ARITH_EXACT))
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout=layout)
    samples = torch.zeros(1, dtype=torch.int64, device="cuda")
    out = api.trace(fs, _dev(xs), _dev(ys), _dev(zs), prm, s_len=0.25, tol_coef=1.0, schedule=sched,
                    samples=samples)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    if layout in ("h4b", "h8c"):
        # fp16 node values (relative rounding up to 2^-12 of the brick's or
        # cell's scale) move footpoints by more than the arithmetic does:
        # within 2e-2 cell on >= 99 %; the arithmetic alone is held to the
        # float32 bars in test_fp16_stores_arithmetic_parity
        check_parity(got, ref, flag_frac=0.998, foot_frac=0.99, tol=2e-2)
    else:
        check_parity(got, ref, flag_frac=0.998, foot_frac=0.99)
    assert int(samples.item()) > 6 * len(xs)


@pytest.mark.parametrize("layout,arith", [("f4", P.ARITH_FAST), ("h4b", P.ARITH_FAST), ("h8c", P.ARITH_FAST),
                                          ("h4b", P.ARITH_FAST_W16)])
def test_fp16_stores_arithmetic_parity(cuda, oracle_port, layout, arith):
    """On a field the fp16 stores hold exactly (golden_util.fp16_exact_field)
    the fp16 stores' FP32 interpolation traces like the float32 store: the
    same bars as the interleaved float32 store (flags >= 99.8 %, footpoints
    within 1e-3 cell on >= 99 %) against the FP32 oracle of the reference's
    tracer on the same field.  The opt-in fp16-x-weight sampler quantises the
    x fraction to ~2^-11 and is held to its own, looser bar (flags >= 99 %,
    footpoints within 2e-2 cell on >= 98 %)."""
    from fastqsl_gb300 import api, synthetic as S
    B = G.fp16_exact_field(S.make_field(S.charges_random(3, (96, 96, 64), 8)))
    xs, ys, zs, shp = S.plane_seeds((2, 93), (2, 93), 72, 72, 0.5)
    ref = oracle_port.trace_all("port32", *B, xs, ys, zs, s_len=0.25, tol_coef=1.0,
                                params=P.absolute_rkf45(arith=P.ARITH_EXACT))
    fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout=layout)
    out = api.trace(fs, _dev(xs), _dev(ys), _dev(zs), P.absolute_rkf45(arith=arith), s_len=0.25, tol_coef=1.0,
                    schedule="queue")
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    if arith == P.ARITH_FAST_W16:
        check_parity(got, ref, flag_frac=0.99, foot_frac=0.98, tol=2e-2)
    else:
        check_parity(got, ref, flag_frac=0.998, foot_frac=0.99)


def test_w16_rejected_off_the_brick_store(cuda):
    """fp16 x weights are a sampler of the brick store: other layouts refuse
    them with a clear error."""
    from fastqsl_gb300 import api, _lib, synthetic as S
    B = S.make_field(S.bipole4_64(0))
    fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout="f4")
    x = torch.full((4,), 10.0, device="cuda")
    with pytest.raises(_lib.QslError, match="h4b"):
        api.trace(fs, x, x, x, P.absolute_rkf45(arith=P.ARITH_FAST_W16))


def test_edge_seeds(cuda, oracle_port):
    """Seeds on faces, edges and outside the box, a NaN seed, an empty call."""
    from fastqsl_gb300 import api, synthetic as S
    spec = S.bipole4_64(2)
    Bx, By, Bz = S.make_field(spec)
    pts = np.array([[0, 0, 0], [63, 63, 63], [0, 30, 10], [63, 10, 5], [10, 0, 5], [10, 63, 5], [20, 20, 63],
                    [-1, 5, 5], [70, 5, 5], [5, 5, -3], [np.nan, 5, 5], [31.5, 31.5, 0], [1e-7, 1e-7, 1e-7]],
                   dtype=np.float32)
    xs, ys, zs = pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy()
    for kind, prm, sl in (("rk4", P.reference_rk4(), 0.1), ("rkf45", P.reference_rkf45(), 0.125)):
        ref = oracle_port.trace_all("port32cr", Bx, By, Bz, xs, ys, zs, s_len=sl, params=prm)
        got = run_dropin(kind, Bx, By, Bz, xs, ys, zs, sl, 1.0)
        np.testing.assert_array_equal(got["flag_start"], ref["flag_start"])
        np.testing.assert_array_equal(got["flag_end"], ref["flag_end"])
        fin = np.isfinite(ref["end_x"]) & np.isfinite(ref["start_x"])
        for k in ["end_x", "end_y", "end_z", "start_x", "start_y", "start_z"]:
            np.testing.assert_allclose(got[k][fin], ref[k][fin], atol=1e-4, err_msg=k)
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout="soa")
    e = torch.zeros(0, dtype=torch.float32, device="cuda")
    out = api.trace(fs, e, e, e, P.reference_rkf45())
    torch.cuda.synchronize()
    assert out["flag_end"].numel() == 0


def test_zero_field_terminates(cuda):
    """B = 0 everywhere: b = 0/0 is NaN, positions go NaN, flag 42."""
    from fastqsl_gb300 import api
    z = torch.zeros((16, 16, 16), dtype=torch.float32)
    fs = api.FieldStore(z, z, z, layout="soa")
    xs = torch.tensor([3.0, 7.5], device="cuda")
    for prm in (P.reference_rk4(), P.reference_rkf45(), P.absolute_rkf45()):
        out = api.trace(fs, xs, xs, xs, prm)
        torch.cuda.synchronize()
        assert (out["flag_end"].cpu() == 42).all()
        assert (out["flag_start"].cpu() == 42).all()


@pytest.mark.parametrize("layout,packed", [("soa", False), ("f4", False), ("h4b", False), ("f4", True),
                                           ("h4b", True)])
def test_native_twist_vs_fp64_oracle(cuda, oracle_port, layout, packed):
    """The twist integral of the fast kernels (current density J = curl B
    stand-in, sampled on the traced grid; from the caller's arrays or, packed,
    from a store of the field's layout) against the FP64 oracle, on lines
    whose two exit faces agree; fp16 field storage widens the bar.  A float32
    packed current gives the same integral as the arrays, bit for bit."""
    from fastqsl_gb300 import api, synthetic as S
    spec = S.charges_random(3, (96, 96, 64), 8)
    Bx, By, Bz = S.make_field(spec)
    cur = G.twist_current(Bx, By, Bz)
    xs, ys, zs, shp = S.plane_seeds((2, 93), (2, 93), 48, 48, 0.5)
    prm = P.absolute_rkf45(arith=P.ARITH_FAST)
    ref = oracle_port.trace_all("port64", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0,
                                params=P.absolute_rkf45(arith=P.ARITH_EXACT), curB=cur)
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout=layout)
    curd = _field_dev(*cur)
    if packed:
        cs = api.FieldStore(*curd, layout=layout)
        out = api.trace(fs, _dev(xs), _dev(ys), _dev(zs), prm, s_len=0.25, tol_coef=1.0, schedule="static",
                        curB=cs)
        if layout == "f4":
            arrays = api.trace(fs, _dev(xs), _dev(ys), _dev(zs), prm, s_len=0.25, tol_coef=1.0, schedule="static",
                               curB=curd)
            assert torch.equal(arrays["twist"], out["twist"])
    else:
        out = api.trace(fs, _dev(xs), _dev(ys), _dev(zs), prm, s_len=0.25, tol_coef=1.0, schedule="static",
                        curB=curd)
    torch.cuda.synchronize()
    tw = out["twist"].cpu().numpy()
    same = ((out["flag_start"].cpu().numpy() == ref["flag_start"]) & (out["flag_end"].cpu().numpy() == ref["flag_end"])
            & (ref["flag_start"] != 0) & (ref["flag_end"] != 0))
    assert same.mean() > 0.9
    rel = np.abs(tw[same] - ref["twist"][same]) / np.maximum(np.abs(ref["twist"][same]), 1e-3)
    med, p90 = np.median(rel), np.quantile(rel, 0.9)
    ll = out["LineLen"].cpu().numpy()
    rl = np.abs(ll[same] - ref["LineLen"][same]) / np.maximum(ref["LineLen"][same], 1e-6)
    print(layout, packed, "twist rel err median %.2e p90 %.2e" % (med, p90), "len rel median %.2e p90 %.2e" % (
        np.median(rl), np.quantile(rl, 0.9)))
    # fp16 bricks: the node values' rounding moves the step sequence a
    # little, and the twist is a first-order sum over the steps (the
    # reference's rule)
    bar = (1e-3, 1e-2) if layout == "h4b" else (1e-4, 1e-3)
    assert med <= bar[0] and p90 <= bar[1], (med, p90)


def test_qmap_plan_twist_map(cuda):
    """QMapPlan.run with a current density: Q unchanged, and each seed's twist
    equal to the single trace's (the plan's tile order only reassigns lines
    to threads)."""
    from fastqsl_gb300 import api, synthetic as S
    spec = S.charges_random(4, (64, 56, 48), 6)
    B = S.make_field(spec)
    cur = G.twist_current(*B)
    fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout="h4b")
    cs = api.FieldStore(*_field_dev(*cur), layout="h4b")
    n0, n1 = 20, 24
    xs, ys, zz = api.plane_seed_grid(4.0, 4.0 + 2.0 * (n1 - 1), n1, 4.0, 4.0 + 2.0 * (n0 - 1), n0, [0.5, 3.0])
    prm = P.absolute_rkf45(arith=P.ARITH_FAST)
    plan = api.QMapPlan(n0, n1, 2)
    assert plan.twist_map is None
    Q0 = plan.run(fs, xs, ys, zz, prm, s_len=0.25, stride=2.0).clone()
    Q1 = plan.run(fs, xs, ys, zz, prm, s_len=0.25, stride=2.0, curB=cs)
    assert torch.equal(torch.nan_to_num(Q0, nan=-1.0), torch.nan_to_num(Q1, nan=-1.0))
    ref = api.trace(fs, xs, ys, zz, prm, s_len=0.25, schedule="static", curB=cs, occupancy=plan.occupancy_for(fs))
    assert plan.twist_map.shape == (2, n0, n1)
    assert torch.equal(plan.twist_map.reshape(-1), ref["twist"])


def test_line_status(cuda):
    """Each direction's qsl_line_status (the reference reports only flag 0 for
    every limit and 42 for edges and non-finite positions alike):
    * faces (flags 1-6) on an ordinary field, EDGE for a flag-42 exit at a
      finite position (two coordinates crossing their faces in one step);
    * MAX_STEPS (max_steps = 5) and MAX_LENGTH (a length limit of ~2 cells),
      flag 0, footpoint where the line stopped;
    * REJECT_LIMIT with a tolerance no step meets (1e-30) and max_rejects 5:
      flag 0, and for most lines the seed itself as footpoint; with tol = 0
      and no reject
      limit the controller rejects until the step size underflows and the
      position turns non-finite: NAN, flag 42;
    * NAN for lines started in a cell with an infinite node value."""
    from fastqsl_gb300 import api, synthetic as S
    B = S.make_field(S.bipole4_64(0))
    xs, ys, zs, _ = S.plane_seeds((4, 59), (4, 59), 24, 24, 0.5)
    x, y, z = _dev(xs), _dev(ys), _dev(zs)
    for layout, arith in (("soa", P.ARITH_EXACT), ("h4b", P.ARITH_FAST), ("f4", P.ARITH_FAST)):
        fs = api.FieldStore(*[torch.from_numpy(b) for b in B], layout=layout)
        base = P.absolute_rkf45(arith=arith)

        def run(prm, sx=x, sy=y, sz=z):
            o = api.trace(fs, sx, sy, sz, prm, s_len=0.25, status=True)
            torch.cuda.synchronize()
            return {k: v.cpu().numpy() for k, v in o.items() if v is not None}

        o = run(base)
        for f, st in (("flag_start", "status_start"), ("flag_end", "status_end")):
            face = (o[f] >= 1) & (o[f] <= 6)
            assert face.mean() > 0.9
            assert (o[st][face] == P.LINE_FACE).all()
            assert (o[st][o[f] == 42] == P.LINE_EDGE).all()
        for prm, want in ((base.copy(max_steps=5), P.LINE_MAX_STEPS), (base.copy(len_ratio=0.01),
                                                                        P.LINE_MAX_LENGTH)):
            o = run(prm)
            st = np.concatenate([o["status_start"], o["status_end"]])
            fl = np.concatenate([o["flag_start"], o["flag_end"]])
            assert ((st == want) == (fl == 0)).all()
            assert (st == want).mean() > 0.4
            assert np.isfinite(o["end_x"]).all() and np.isfinite(o["start_x"]).all()
        o = run(base.copy(tol=1e-30, max_rejects=5))
        for f, st, k in (("flag_start", "status_start", "start_x"), ("flag_end", "status_end", "end_x")):
            assert (o[st] == P.LINE_REJECT_LIMIT).all() and (o[f] == 0).all()
            # a step is accepted only where its error estimate is exactly 0
            # (every stage samples the same clamped value past a face): most
            # lines end where they started
            assert (o[k] == xs).mean() > 0.9
        o = run(base.copy(tol=0.0, max_rejects=0))
        assert (o["status_end"] == P.LINE_NAN).all() and (o["flag_end"] == 42).all()
        fs.close()
    # edge exit: B along (1, 1, 0), seeds on the diagonal near the x-max / y-max edge
    one = np.ones((32, 32, 32), np.float32)
    fs = api.FieldStore(torch.from_numpy(one), torch.from_numpy(one), torch.from_numpy(0 * one), layout="f4")
    e = torch.tensor([29.5, 30.25], device="cuda")
    o = api.trace(fs, e, e, torch.full_like(e, 7.0), P.absolute_rkf45(), s_len=0.25, status=True)
    torch.cuda.synchronize()
    assert (o["flag_end"].cpu() == 42).all() and (o["status_end"].cpu() == P.LINE_EDGE).all()
    assert torch.isfinite(o["end_x"]).all()
    fs.close()
    # poisoned field: an infinite node in the seeds' cell
    Bp = [b.copy() for b in B]
    Bp[0][20, 20, 0] = np.inf
    fs = api.FieldStore(*[torch.from_numpy(b) for b in Bp], layout="f4")
    p = torch.tensor([20.25, 19.5], device="cuda")
    o = api.trace(fs, p, torch.tensor([20.5, 19.75], device="cuda"), torch.tensor([0.5, 0.25], device="cuda"),
                  P.absolute_rkf45(), s_len=0.25, status=True)
    torch.cuda.synchronize()
    assert (o["status_end"].cpu() == P.LINE_NAN).all() and (o["flag_end"].cpu() == 42).all()
    fs.close()
