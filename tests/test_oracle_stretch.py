"""The stretched-grid oracle (oracle/port/qsl_port.c, trace_all_stretch)
pinned to the reference's own TraceBlineAdaptiveStretch.cu:

* against the golden fixtures made from the reference's host build
  (tests/golden/make_golden.py): every output bit for bit, except the
  footpoints of directions stopped by the length limit (the reference reports
  stale scratch memory there);
* against a fresh reference build where the reference checkout exists:
  the index search, the uniform-spacing index formula, the interpolation and
  the boundary test on random points.
"""
import numpy as np
import pytest

import oracle
from fastqsl_gb300 import params as P, synthetic as S
import golden_util as G


def _same(a, b):
    return (a == b) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("name", G.STRETCH_CASES)
def test_port32_matches_reference_stretch(oracle_port, name):
    g, meta = G.load(name)
    Bx, By, Bz, coords = G.stretch_field_for(meta)
    for c, k in zip(coords, ("xa", "ya", "za")):
        np.testing.assert_array_equal(c, g[k])
    cur = G.twist_current(Bx, By, Bz) if meta["twist"] else None
    got = oracle.trace_all("port32", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], s_len=meta["s_len"],
                           tol_coef=meta["tol_coef"], params=P.reference_stretch(), curB=cur, coords=coords,
                           uni=meta["uni"])
    for k in ("flag_start", "flag_end", "B_flag", "B_this_x", "B_this_y", "B_this_z", "LineLen"):
        assert _same(got[k], g[k]).all(), k
    if meta["twist"]:
        # A direction whose exit step is shorter than 1e-3 along the exit axis
        # ends at its last inside point, and the reference's exit-segment twist
        # term then reads an uninitialised p_mid
        # (TraceBlineAdaptiveStretch.cu:375-404); the oracle adds 0.  Every
        # other exit ends on the plane q = 0 (min face) or q = n (max face) of
        # the exit axis, which identifies the short exits.
        short = np.zeros(len(g["flag_end"]), bool)
        for side in ("start", "end"):
            fl = g["flag_" + side]
            for d, ax in enumerate("xyz"):
                for odd, q in ((True, 0.0), (False, float(Bx.shape[d]))):
                    m = (fl >= 1) & (fl <= 6) & ((fl - 1) // 2 == d) & ((fl % 2 == 1) == odd)
                    short |= m & (np.abs(g[f"{side}_{ax}"] - q) > 1e-6 * max(1.0, abs(q)))
        assert short.mean() < 0.05
        assert _same(got["twist"], g["twist"])[~short].all()
    live_e, live_s = g["flag_end"] != 0, g["flag_start"] != 0
    for k in ("end_x", "end_y", "end_z", "B_end_x", "B_end_y", "B_end_z"):
        assert _same(got[k], g[k])[live_e].all(), k
    for k in ("start_x", "start_y", "start_z", "B_start_x", "B_start_y", "B_start_z"):
        assert _same(got[k], g[k])[live_s].all(), k
    assert live_e.mean() > 0.9 and live_s.mean() > 0.9


@pytest.mark.skipif(not oracle.ref_available("stretch"), reason="reference host build not present")
@pytest.mark.parametrize("z_ratio", [1.06, 1.0])
def test_port32_stretch_probes_match_reference_build(oracle_port, z_ratio):
    spec = S.bipole4_stretch(4)
    xa, ya, za = S.stretched_axes(spec.shape, z_ratio=z_ratio)
    Bx, By, Bz = S.make_field_coords(spec, xa, ya, za)
    rng = np.random.default_rng(11)
    pts = np.stack([rng.uniform(-7, 7, 600), rng.uniform(-6, 6, 600), rng.uniform(-1, 11, 600)], 1)
    pts = pts.astype(np.float32)
    pts[:60, 2] = za[rng.integers(0, za.size, 60)]  # on nodes
    pts[60:80, 0] = xa[0]
    pts[80:100, 1] = ya[-1]
    for uni in (False, True):
        mine = oracle.StretchProbe("port32", Bx, By, Bz, (xa, ya, za), uni)
        ref = oracle.StretchProbe("ref_stretch", Bx, By, Bz, (xa, ya, za), uni)
        for p in pts:
            for ax in range(3):
                assert mine.index(p[ax], ax) == ref.index(p[ax], ax)
            for unit in (True, False):
                assert _same(mine.interp(p, unit), ref.interp(p, unit)).all()
            assert mine.checkflag(p) == ref.checkflag(p)


def test_reference_search_can_pick_the_cell_below():
    """The reference's search returns the cell below the point for points in
    the upper part of its last 3-node interval (restated as is): on 16 unit
    nodes, 10.5 lands in cell 9."""
    a = np.arange(16, dtype=np.float32)
    pr = oracle.port_lib()
    import ctypes
    f = pr.qo32_index_bisect
    ptr = a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert f(ctypes.c_float(7.5), 16, ptr) == 7
    assert f(ctypes.c_float(10.5), 16, ptr) == 9
