"""The MagTool restatement (oracle/magtool.py) pinned to the reference's own
fastqslpy/MagTool.py: the golden fixture holds its TraceBline polylines and
its trilerp / Bnorm values (tests/golden/make_golden.py magtool); the
restatement reproduces every one bit for bit."""
import numpy as np

import golden_util as G
from oracle import magtool as M


def _same(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_trace_bline_matches_reference():
    g, B = G.magtool_case()
    npts = []
    for seed, ref in zip(g["seeds"], g["lines"]):
        got = np.stack(M.trace_bline(B, seed, 800))
        assert _same(got, ref)
        npts.append(int((~np.isnan(ref[0])).sum()))
    # the fixture covers long lines, lines along the clamped top plane and a
    # seed on the box corner
    assert max(npts) > 300 and min(npts) == 1
    top = g["lines"][7]
    assert np.nanmax(top[2]) == 24.0 and np.nanmax(top[0]) > 39.9


def test_trilerp_bnorm_match_reference():
    g, B = G.magtool_case()
    for p, t, b in zip(g["pts"], g["trilerp"], g["bnorm"]):
        assert np.array_equal(M.trilerp(B, p), t)
        assert np.array_equal(M.bnorm(B, p), b)
