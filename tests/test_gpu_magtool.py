"""The MagTool drop-in (fastqsl_gb300.fastqslpy.MagTool, kernels
qsl_trace_path / qsl_sample_points) against the reference's own MagTool
outputs (golden fixture) and the restatement in oracle/magtool.py: float64
arithmetic in the reference's order, so every stored point and every sample
is compared for equality."""
import numpy as np
import pytest
import torch

import golden_util as G

pytestmark = pytest.mark.gpu


def _same(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_trace_bline_bitexact_vs_reference(cuda):
    from fastqsl_gb300.fastqslpy import MagTool as mt
    g, B = G.magtool_case()
    for seed, ref in zip(g["seeds"], g["lines"]):
        p = seed.copy()
        lx, ly, lz = mt.TraceBline(*B, p, dr=0.25, maxstep=800)
        assert lx.dtype == np.float32 and lx.shape == (800,)
        assert _same(np.stack([lx, ly, lz]), ref)
    # many seeds in one launch pair: the same lines
    xs, ys, zs = mt.TraceBlines(*B, g["seeds"], maxstep=800, dr=0.25)
    assert _same(np.stack([xs, ys, zs], 1), g["lines"])


def test_trilerp_bnorm_bitexact_vs_reference(cuda):
    from fastqsl_gb300.fastqslpy import MagTool as mt
    g, B = G.magtool_case()
    for p, t, b in zip(g["pts"], g["trilerp"], g["bnorm"]):
        assert np.array_equal(mt.trilerp(*B, p.copy()), t)
        assert np.array_equal(mt.Bnorm(*B, p.copy()), b)
    # in-place clamp of the caller's point, as the reference's trilerp does
    v = np.array([-1.0, 40.0, 30.0])
    mt.trilerp(*B, v)
    assert v[0] == 1e-8 and v[1] == 32 - 1e-8 and v[2] == 24 - 1e-8
    # all points at once, device field
    Bd = [torch.from_numpy(b).cuda() for b in B]
    np.testing.assert_array_equal(mt.Bnorm(*Bd, g["pts"]), g["bnorm"])


def test_rk4_bline_ranges_vs_oracle(cuda):
    """RK4_bline into caller arrays over strided and reversed ranges and
    steps other than 0.25; entries outside the range keep their values."""
    from fastqsl_gb300.fastqslpy import MagTool as mt
    from oracle import magtool as M
    g, B = G.magtool_case()
    for seed, rng, dr in ((g["seeds"][0], range(10, 700, 3), 0.4), (g["seeds"][3], range(600, 4, -2), -0.3),
                          (g["seeds"][5], range(0, 0), 0.25)):
        ref = [np.arange(800, dtype=np.float32) for _ in range(3)]
        got = [a.copy() for a in ref]
        M.rk4_bline(B, seed, *ref, rng, dr)
        mt.RK4_bline(*B, seed.copy(), *got, rng, dr=dr)
        for a, b in zip(got, ref):
            assert _same(a, b)


def test_trace_path_rejects_out_of_range_rows(cuda):
    from fastqsl_gb300 import _lib
    from fastqsl_gb300.api import stream_handle
    B = [torch.zeros((4, 4, 4), device="cuda") for _ in range(3)]
    s = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros((3, 10), dtype=torch.float32, device="cuda")
    lib = _lib.load()
    args = [b.data_ptr() for b in B] + [4, 4, 4, s.data_ptr(), 1]
    tail = [0.25, out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), 10, stream_handle()]
    assert lib.qsl_trace_path(*args, 5, 11, 1, *tail) != 0       # index 10 is past the row
    assert lib.qsl_trace_path(*args, 5, -2, -1, *tail) != 0      # index -1
    assert lib.qsl_trace_path(*args, 0, 5, 0, *tail) != 0        # zero stride
    assert lib.qsl_trace_path(*args, 9, -1, -3, *tail) == 0      # 9, 6, 3, 0
    torch.cuda.synchronize()
