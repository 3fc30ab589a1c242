"""The CPU oracle against the reference's own outputs (golden fixtures made
by running the reference code; see tests/golden/make_golden.py).

The FP32 restatement must reproduce the reference bit for bit, except in
the places where the reference reads uninitialised memory (footpoints of
directions stopped by a limit; the RK4 exit-segment twist term when the exit
step is shorter than 1e-3; the Scott routine's outputs of lines it leaves
unset)."""
import numpy as np
import pytest

import golden_util as G
from fastqsl_gb300 import params as P


def _params(kind):
    return P.reference_rk4() if kind == "rk4" else P.reference_rkf45()


@pytest.mark.parametrize("name", sorted(G.TRACE_CASES))
def test_port32_matches_reference_trace(oracle_port, name):
    g, meta = G.load(name)
    kind, twist = G.TRACE_CASES[name]
    Bx, By, Bz = G.field_for(meta)
    cur = G.twist_current(Bx, By, Bz) if twist else None
    out = oracle_port.trace_all("port32", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], s_len=meta["s_len"],
                                tol_coef=meta["tol_coef"], params=_params(kind), curB=cur)
    ok = G.limit_mask(g)
    for k in ["flag_start", "flag_end", "B_flag", "B_this_x", "B_this_y", "B_this_z", "LineLen"]:
        np.testing.assert_array_equal(out[k], g[k], err_msg=k)
    for k in G.FOOT_KEYS:
        np.testing.assert_array_equal(out[k][ok], g[k][ok], err_msg=k)
    if twist:
        same = out["twist"] == g["twist"]
        if kind == "rkf45":
            assert same.all()
        else:
            # the reference's RK4 exit-segment twist term reads p_mid
            # uninitialised when the exit step is < 1e-3 in the normal
            # coordinate; those lines end within 1e-3 of a face
            assert same.mean() > 0.99
            near_face = (np.minimum(np.abs(g["start_z"]), np.abs(g["end_z"])) < 1.5e-3)
            assert near_face[~same].all()


def test_port32_matches_reference_probes(oracle_port):
    g, meta = G.load("probes_bipole4_64.npz")
    Bx, By, Bz = G.field_for(meta)
    pr = oracle_port.Probe("port32", Bx, By, Bz)
    pts, hs, dims, v9 = g["pts"], g["hs"], g["dims"], g["v9"]
    np.testing.assert_array_equal(np.stack([pr.interp(p, True) for p in pts]), g["interp_unit"])
    np.testing.assert_array_equal(np.stack([pr.interp(p, False) for p in pts]), g["interp_raw"])
    np.testing.assert_array_equal(np.array([[pr.interp_scalar(c, p) for c in range(3)] for p in pts], np.float32),
                                  g["interp_scalar"])
    np.testing.assert_array_equal(np.array([pr.checkflag(p) for p in pts]), g["checkflag"])
    np.testing.assert_array_equal(np.stack([pr.rk4(p, h) for p, h in zip(pts, hs)]), g["rk4"])
    np.testing.assert_array_equal(np.stack([pr.rkf45(p, h) for p, h in zip(pts, hs)]), g["rkf45"])
    np.testing.assert_array_equal(np.stack([pr.rk4_boundary(p, h, int(d)) for p, h, d in zip(pts, hs, dims)]),
                                  g["rk4_boundary"])
    np.testing.assert_array_equal(np.stack([pr.grad_unit_b(p) for p in pts]), g["grad_unit_b"])
    np.testing.assert_array_equal(np.stack([pr.f_scott(v) for v in v9]), g["f_scott"])
    sc = [pr.rkf45_scott(v, h) for v, h in zip(v9, hs)]
    np.testing.assert_array_equal(np.stack([s[0] for s in sc]), g["rkf45_scott"])
    np.testing.assert_array_equal(np.array([s[1] for s in sc], np.float32), g["rkf45_scott_err"])


@pytest.mark.parametrize("name", sorted(G.SCOTT_CASES))
def test_port32_matches_reference_scott_lines(oracle_port, name):
    """Whole Scott lines (TraceBlineScott.cu:334-519, the reference built with
    its tolerance initialised): exit faces of every seed the reference
    defines, footpoints, q_0, q_perp, B at the seed and (twist on) the twist
    integral, bit for bit."""
    g, meta = G.load(name)
    Bx, By, Bz = G.field_for(meta)
    cur = G.twist_current(Bx, By, Bz) if meta["twist"] else None
    out = oracle_port.scott_all("port32", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], s_len=meta["s_len"],
                                tol_coef=meta["tol_coef"], params=P.reference_scott(), curB=cur)
    live = G.scott_live(g)
    assert live.mean() > 0.85
    defined = g["inp_z"] >= 0
    for k in ["flag_start", "flag_end"]:
        np.testing.assert_array_equal(out[k][defined], g[k][defined], err_msg=k)
    for k in ["B_this_x", "B_this_y", "B_this_z"]:
        np.testing.assert_array_equal(out[k][defined], g[k][defined], err_msg=k)
    for k in ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z", "q_0", "q_perp"] + (
            ["twist"] if meta["twist"] else []):
        np.testing.assert_array_equal(out[k][live], g[k][live], err_msg=k)


def test_qassembly_matches_reference(oracle_port):
    from oracle import qassembly as QA
    g, meta = G.load("qmap_rkf45_bipole4_64.npz")
    shp = tuple(meta["xy_shape"])
    r = lambda k: g["main_" + k].reshape(shp)  # noqa: E731
    stride = 1 / meta["interp_ratio"]
    Q = QA.qcalc_plane(r("end_x"), r("end_y"), r("end_z"), r("flag_end"), r("start_x"), r("start_y"),
                       r("start_z"), r("flag_start"), r("B_start_x"), r("B_start_y"), r("B_start_z"),
                       r("B_end_x"), r("B_end_y"), r("B_end_z"), r("B_this_x"), r("B_this_y"), r("B_this_z"),
                       r("B_flag"), stride)
    np.testing.assert_array_equal(Q, g["Q"])
    cx, cy, cz, bzs, bze = QA.cook_pseudo_line(r("start_x"), r("start_y"), r("start_z"), r("flag_start"),
                                               r("B_start_z"), r("B_end_z"), r("B_flag"), np.float32(stride))
    for a, k in ((cx, "cut_inp_x"), (cy, "cut_inp_y"), (cz, "cut_inp_z"), (bzs, "Bz0_start"), (bze, "Bz0_end")):
        np.testing.assert_array_equal(a, g[k], err_msg=k)
    c = lambda k: g["cut_" + k]  # noqa: E731
    Qc = QA.qcut(c("start_x"), c("start_y"), c("start_z"), c("flag_start"), c("end_x"), c("end_y"), c("end_z"),
                 c("flag_end"), g["Bz0_start"], g["Bz0_end"], np.float32(stride))
    np.testing.assert_array_equal(Qc, g["Qcut"])
    _, Qf = QA.merge(Q, Qc, r("B_flag"))
    np.testing.assert_array_equal(Qf, g["Q_final"])


def test_pseudo_line_trace_matches_reference(oracle_port):
    """The second (pseudo-line) trace of the Q-map workflow, on seeds that sit
    on the boundary faces."""
    g, meta = G.load("qmap_rkf45_bipole4_64.npz")
    Bx, By, Bz = G.field_for(meta)
    out = oracle_port.trace_all("port32", Bx, By, Bz, g["cut_inp_x"], g["cut_inp_y"], g["cut_inp_z"],
                                s_len=meta["s_len"], tol_coef=np.float32(meta["tol_coef"] * 0.1),
                                params=P.reference_rkf45())
    ok = (g["cut_flag_start"] != 0) & (g["cut_flag_end"] != 0)
    for k in ["flag_start", "flag_end", "LineLen"]:
        np.testing.assert_array_equal(out[k], g["cut_" + k], err_msg=k)
    for k in ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z"]:
        np.testing.assert_array_equal(out[k][ok], g["cut_" + k][ok], err_msg=k)


@pytest.mark.skipif(not __import__("oracle").ref_available("rkf45"), reason="reference host build not present")
@pytest.mark.parametrize("kind", ["rk4", "rkf45"])
def test_port32_matches_reference_build_fresh(oracle_port, kind):
    """Against the reference compiled from its sources (where it exists), on
    a field and seeds the fixtures do not contain."""
    from fastqsl_gb300 import synthetic as S
    spec = S.charges_random(11, (40, 36, 30), 6)
    Bx, By, Bz = S.make_field(spec)
    rng = np.random.default_rng(5)
    n = 1500
    xs = rng.uniform(0, 39, n).astype(np.float32)
    ys = rng.uniform(0, 35, n).astype(np.float32)
    zs = rng.uniform(0, 29, n).astype(np.float32)
    sl = 0.1 if kind == "rk4" else 0.125
    ref = oracle_port.trace_all("ref_" + kind, Bx, By, Bz, xs, ys, zs, cross_dir=(0.3, -0.2, 0.93), s_len=sl,
                                tol_coef=0.7)
    out = oracle_port.trace_all("port32", Bx, By, Bz, xs, ys, zs, cross_dir=(0.3, -0.2, 0.93), s_len=sl,
                                tol_coef=0.7, params=_params(kind))
    ok = G.limit_mask(ref)
    for k in ["flag_start", "flag_end", "B_flag", "LineLen", "B_this_x"]:
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    for k in G.FOOT_KEYS:
        np.testing.assert_array_equal(out[k][ok], ref[k][ok], err_msg=k)


def test_fp64_oracle_close_to_fp32_on_smooth_lines(oracle_port):
    """The FP64 oracle runs the same algorithm: on lines that end on the
    same face, footpoints agree to well under a cell."""
    g, meta = G.load("trace_rkf45_bipole4_64.npz")
    Bx, By, Bz = G.field_for(meta)
    prm = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=P.ARITH_EXACT)
    a = oracle_port.trace_all("port32", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], params=prm)
    b = oracle_port.trace_all("port64", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], params=prm)
    same = (a["flag_end"] == b["flag_end"]) & (a["flag_start"] == b["flag_start"])
    assert same.mean() > 0.99
    d = np.hypot(a["end_x"] - b["end_x"], a["end_y"] - b["end_y"])[same & (a["flag_end"] == 5)]
    assert np.median(d) < 1e-3
