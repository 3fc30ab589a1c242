"""Host-side Q-assembly pieces of the oracle pinned to the reference:

* the hybrid finite-difference + Scott Q merge (oracle/qassembly.py) against
  the reference's own notebook cell that defines it
  (demo/Q_RKF45MixCuPyDiffScott.ipynb cell 9), executed from the notebook file
  with NumPy standing in for CuPy and a stand-in Scott kernel;
* curl B on a stretched grid against the reference's curl_of_B_grid
  (golden fixture made by tests/golden/make_golden.py)."""
import json
import os
import types

import numpy as np
import pytest

from oracle import qassembly as QA

# the reference checkout: $QSL_REFERENCE_ROOT, else `reference` beside the repository
REF = os.environ.get("QSL_REFERENCE_ROOT", os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference"))
NB = os.path.join(REF, "demo", "Q_RKF45MixCuPyDiffScott.ipynb")


class _G(np.ndarray):
    """numpy array with CuPy's .get()"""

    def get(self):
        return np.asarray(self)


def _g(a):
    return np.asarray(a).view(_G)


def _fake_cupy():
    cp = types.SimpleNamespace()
    cp.where = lambda c: tuple(_g(i) for i in np.where(np.asarray(c)))
    cp.isnan = lambda a: _g(np.isnan(np.asarray(a)))
    cp.zeros = lambda shape, dtype=np.float32: _g(np.zeros(shape, dtype))
    cp.array = lambda a, dtype=None: _g(np.array(a, dtype))
    cp.float32, cp.int32, cp.ulonglong = np.float32, np.int32, np.ulonglong
    cp.cuda = types.SimpleNamespace(stream=types.SimpleNamespace(
        get_current_stream=lambda: types.SimpleNamespace(synchronize=lambda: None)))
    return cp


def _q_of_seed(x, y):
    return (1.0 + 1000.0 * np.asarray(x, np.float64) + np.asarray(y, np.float64)).astype(np.float32)


@pytest.mark.skipif(not os.path.exists(NB), reason="reference checkout not present")
def test_hybrid_merge_matches_reference_notebook():
    rng = np.random.default_rng(3)
    n0, n1 = 9, 12
    xy_shape = (n0, n1)
    x_inp = _g(np.tile(np.arange(n1, dtype=np.float32), n0))
    y_inp = _g(np.repeat(np.arange(n0, dtype=np.float32), n1))
    B_flag = _g((rng.random(n0 * n1) < 0.15).astype(np.int32))
    Q = rng.uniform(1, 100, size=(n0 - 2, n1 - 2))
    Q[rng.random(Q.shape) < 0.2] = np.nan
    Q_all = np.zeros(xy_shape, np.float32)  # as the notebook's cell 7 builds it (edges 0)
    Q_all[1:-1, 1:-1] = Q
    Q_all = _g(Q_all)

    def scott_stub(blck, grd, args):
        args[25][:] = _q_of_seed(args[9], args[10])  # q_perp of the selected seeds (q_0 is args[24])

    f32 = lambda: _g(np.zeros(n0 * n1, np.float32))  # noqa: E731
    ns = dict(cupy=_fake_cupy(), np=np, B_flag=B_flag, Q_all=Q_all, x_inp=x_inp, y_inp=y_inp,
              z_inp=_g(np.zeros(n0 * n1, np.float32)), xy_shape=xy_shape, TraceAllBlineScott=scott_stub,
              blck=(128, 1, 1), grd=(28, 1), Bx_gpu=None, By_gpu=None, Bz_gpu=None, BshapeN=None, dummy=None,
              flag_twist=None, inp_norm=None, s_len=None, line_len=None, real_tol=None, clear_tmp=False,
              x_start=f32(), y_start=f32(), z_start=f32(), x_end=f32(), y_end=f32(), z_end=f32(),
              flag_start=_g(np.zeros(n0 * n1, np.int32)), flag_end=_g(np.zeros(n0 * n1, np.int32)),
              Bx_inp=f32(), By_inp=f32(), Bz_inp=f32(), q_0_gpu=f32(), q_perp_gpu=f32())
    with open(NB) as fh:
        src = "".join(json.load(fh)["cells"][9]["source"])
    exec(compile(src, "Q_RKF45MixCuPyDiffScott.ipynb:cell9", "exec"), ns)
    ref = np.asarray(ns["Q_all_update"], np.float64)[1:-1, 1:-1]
    mine = QA.hybrid_merge(Q, np.asarray(B_flag).reshape(xy_shape),
                           _q_of_seed(np.asarray(x_inp), np.asarray(y_inp)).reshape(xy_shape))
    np.testing.assert_array_equal(mine.astype(np.float32), ref.astype(np.float32))


def test_curl_matches_reference_fixture():
    import golden_util as G
    from fastqsl_gb300 import synthetic as S
    g, meta = G.load("curl_stretch.npz")
    spec = S.bipole4_stretch(meta["seed"], shape=tuple(meta["shape"]))
    xa, ya, za = S.stretched_axes(spec.shape, z_ratio=meta["z_ratio"])
    Bx, By, Bz = S.make_field_coords(spec, xa, ya, za)
    assert S.field_fingerprint(Bx, By, Bz) == meta["fingerprint"]
    for mine, k in zip(QA.curl_grid(Bx, By, Bz, xa, ya, za), ("curl_x", "curl_y", "curl_z")):
        np.testing.assert_array_equal(mine, g[k])
