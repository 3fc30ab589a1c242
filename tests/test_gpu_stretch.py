"""Stretched-grid tracer (fastqslpy/cu/TraceBlineAdaptiveStretch.cu) on the
GPU through the C ABI:

* the drop-in entry in the reference's notebook form (exact arithmetic)
  against the reference's own outputs (golden fixtures) and bit for bit
  against the oracle built with the same correctly rounded power function;
* the native entry in fast arithmetic at tight settings against the FP64
  oracle (flags identical for >= 99 %, footpoints on the bottom face within
  1e-3 for >= 99 %).
"""
import numpy as np
import pytest
import torch

import golden_util as G
from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu

F32 = ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z", "B_this_x", "B_this_y", "B_this_z",
       "B_start_x", "B_start_y", "B_start_z", "B_end_x", "B_end_y", "B_end_z"]
I32 = ["flag_start", "flag_end", "B_flag"]


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _fdev(a):
    from fastqsl_gb300.api import as_xfast
    return as_xfast(torch.from_numpy(np.asfortranarray(a)))


def run_dropin_stretch(Bx, By, Bz, coords, uni, xs, ys, zs, s_len, tol_coef, curB=None, arith="exact"):
    from fastqsl_gb300.fastqslpy import kernels
    k = kernels.compileTraceBlineAdaptiveStretch(arith)
    n = len(xs)
    o = {key: torch.zeros(n, dtype=torch.float32, device="cuda") for key in F32}
    o.update({key: torch.zeros(n, dtype=torch.int32, device="cuda") for key in I32})
    o["LineLen"] = torch.zeros(n, dtype=torch.float64, device="cuda")
    o["twist"] = torch.zeros(n, dtype=torch.float64, device="cuda")
    dummy = torch.zeros((1, 1), dtype=torch.float32, device="cuda")
    cur = [_fdev(c) for c in curB] if curB is not None else [dummy] * 3
    args = (_fdev(Bx), _fdev(By), _fdev(Bz), torch.tensor(list(Bx.shape), dtype=torch.int32, device="cuda"),
            *[_dev(c) for c in coords], torch.tensor([bool(uni)], device="cuda"),
            *cur, o["twist"], torch.tensor([curB is not None], device="cuda"),
            _dev(xs), _dev(ys), _dev(zs), torch.tensor([0, 0, 1.0], dtype=torch.float32, device="cuda"),
            o["start_x"], o["start_y"], o["start_z"], o["flag_start"],
            o["end_x"], o["end_y"], o["end_z"], o["flag_end"],
            o["B_this_x"], o["B_this_y"], o["B_this_z"], o["B_flag"],
            o["B_start_x"], o["B_start_y"], o["B_start_z"],
            o["B_end_x"], o["B_end_y"], o["B_end_z"],
            torch.tensor([s_len], dtype=torch.float32, device="cuda"),
            torch.tensor([n], dtype=torch.int64, device="cuda"), o["LineLen"],
            torch.tensor([tol_coef], dtype=torch.float32, device="cuda"))
    k((28, 1), (128, 1, 1), args)
    torch.cuda.synchronize()
    return {key: v.cpu().numpy() for key, v in o.items()}


@pytest.mark.parametrize("name", G.STRETCH_CASES)
def test_dropin_stretch_exact_matches_reference(cuda, oracle_port, name):
    g, meta = G.load(name)
    Bx, By, Bz, coords = G.stretch_field_for(meta)
    cur = G.twist_current(Bx, By, Bz) if meta["twist"] else None
    got = run_dropin_stretch(Bx, By, Bz, coords, meta["uni"], g["inp_x"], g["inp_y"], g["inp_z"], meta["s_len"],
                             meta["tol_coef"], cur)
    # against the reference's outputs: flags, and footpoints within 1e-3
    # (RKF45's power function rounds differently from the host powf in
    # ~6e-4 of calls)
    flags = ((got["flag_start"] == g["flag_start"]) & (got["flag_end"] == g["flag_end"])).mean()
    assert flags >= 0.999, flags
    live = (g["flag_start"] != 0) & (g["flag_end"] != 0)
    d = np.max(np.abs(np.stack([got[k] - g[k] for k in ("start_x", "start_y", "start_z", "end_x", "end_y",
                                                        "end_z")])), axis=0)
    assert (d[live] <= 1e-3).mean() >= 0.995
    np.testing.assert_array_equal(got["B_this_x"], g["B_this_x"])
    np.testing.assert_array_equal(got["B_flag"], g["B_flag"])
    if cur is not None:  # the reference's own twist (exit-segment terms with an unset p_mid aside)
        close = np.isclose(got["twist"], g["twist"], rtol=1e-4, atol=1e-7)
        assert close[live].mean() >= 0.95, close[live].mean()
    # bit for bit against the oracle with the same power function
    cr = oracle_port.trace_all("port32cr", Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], s_len=meta["s_len"],
                               tol_coef=meta["tol_coef"], params=P.reference_stretch(), curB=cur, coords=coords,
                               uni=meta["uni"])
    assert (got["flag_end"] == cr["flag_end"]).all() and (got["flag_start"] == cr["flag_start"]).all()
    live = (cr["flag_start"] != 0) & (cr["flag_end"] != 0)
    for k in ("end_x", "end_y", "end_z", "start_x", "start_y", "start_z", "B_end_x", "B_start_z"):
        assert (got[k][live] == cr[k][live]).mean() >= 0.999, k
    rel = np.abs(got["LineLen"] - cr["LineLen"]) / np.maximum(cr["LineLen"], 1e-6)
    assert np.median(rel[live]) < 1e-6
    if cur is not None:
        close = np.isclose(got["twist"], cr["twist"], rtol=1e-5, atol=1e-9)
        assert close[live].mean() >= 0.99, close[live].mean()


@pytest.mark.parametrize("uni", [False, True])
def test_native_stretch_fast_vs_fp64_oracle(cuda, oracle_port, uni):
    """The native entry in fast arithmetic (cell search through the tables,
    or the uniform-spacing formula as a reciprocal product) against the FP64
    oracle of the same search."""
    from fastqsl_gb300 import api, synthetic as S
    spec = S.bipole4_stretch(5)
    coords = S.stretched_axes(spec.shape, z_ratio=1.0 if uni else 1.05)
    Bx, By, Bz = S.make_field_coords(spec, *coords)
    xs, ys, zs, _ = S.plane_seeds((-5, 5), (-4, 4), 48, 40, 0.3)
    # tight tolerance: at 1e-5 the FP32 rounding alone already moves 13 % of
    # the footpoints by more than 1e-3 (accept/reject decisions flip); at 1e-7
    # the reference-rounding FP32 oracle tracks FP64 to 1e-3 on > 99.8 %
    prm = P.reference_stretch(arith=P.ARITH_FAST).copy(tol_law=P.TOL_ABSOLUTE, tol=1e-7, h_min=1e-4, h_max=0.25)
    ref = oracle_port.trace_all("port64", Bx, By, Bz, xs, ys, zs, s_len=0.01, params=prm.copy(arith=P.ARITH_EXACT),
                                coords=coords, uni=uni)
    samples = torch.zeros(1, dtype=torch.int64, device="cuda")
    out = api.trace_stretch(*[torch.from_numpy(np.asfortranarray(b)) for b in (Bx, By, Bz)],
                            [torch.from_numpy(c).cuda() for c in coords], _dev(xs), _dev(ys), _dev(zs), prm,
                            s_len=0.01, samples=samples, uni=uni)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    flags = ((got["flag_start"] == ref["flag_start"]) & (got["flag_end"] == ref["flag_end"])).mean()
    assert flags >= 0.99, flags
    # Footpoints on the bottom face (flag 5): there the reference's exit plane
    # q = 0 (index units) is the physical face z = 0.  Exits through the other
    # faces are projected onto index-unit planes that lie inside or far
    # outside the box (TraceBlineAdaptiveStretch.cu:375-400), a long RK4 leg
    # whose end moves with any rounding.
    for side in ("start", "end"):
        m = (ref[f"flag_{side}"] == 5) & (got[f"flag_{side}"] == 5)
        assert m.mean() > 0.5
        d = np.max(np.abs(np.stack([got[f"{side}_{a}"] - ref[f"{side}_{a}"] for a in "xyz"])), axis=0)
        assert (d[m] <= 1e-3).mean() >= 0.99, (side, np.quantile(d[m], [0.5, 0.99]))
    assert int(samples.item()) > 6 * len(xs)


@pytest.mark.parametrize("uni,twist", [(False, False), (True, True), (False, True)])
def test_native_fast_packed_equals_dropin_fast(cuda, uni, twist):
    """The native stretched entry in fast arithmetic reads the nodes from an
    interleaved float4 copy and finds cells through its search tables, the
    drop-in reads the caller's three arrays and runs the reference's
    search: the same float values, the same cells and the same arithmetic,
    so every output is the same bit for bit (twist included: the current
    stays the caller's arrays)."""
    from fastqsl_gb300 import api, synthetic as S
    spec = S.bipole4_stretch(7)
    coords = S.stretched_axes(spec.shape, z_ratio=1.0 if uni else 1.05)
    Bx, By, Bz = S.make_field_coords(spec, *coords)
    cur = G.twist_current(Bx, By, Bz) if twist else None
    xs, ys, zs, _ = S.plane_seeds((-5, 5), (-4, 4), 40, 32, 0.3)
    got_d = run_dropin_stretch(Bx, By, Bz, coords, uni, xs, ys, zs, 0.01, 1.0, curB=cur, arith="fast")
    prm = P.reference_stretch(arith=P.ARITH_FAST)
    out = api.trace_stretch(*[torch.from_numpy(np.asfortranarray(b)) for b in (Bx, By, Bz)],
                            [torch.from_numpy(c).cuda() for c in coords], _dev(xs), _dev(ys), _dev(zs), prm,
                            s_len=0.01, uni=uni, curB=[_fdev(c) for c in cur] if twist else None)
    torch.cuda.synchronize()
    got_n = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    keys = F32 + I32 + ["LineLen"] + (["twist"] if twist else [])
    for k in keys:
        a, b = got_n[k], got_d[k]
        assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)]), k


@pytest.mark.parametrize("shape", [(4, 3, 5), (2, 4, 4), (5, 2, 3), (4, 4, 4)])
def test_native_tables_equal_dropin_search_on_small_grids(cuda, shape):
    """Axes of 2-5 nodes with irregular spacing: the reference's search takes
    its special cases there (with 4 nodes it answers the cell above for the
    first interval); the native entry's tables must give the same cells.
    Seeds at random points and exactly on node coordinates; every output
    bit for bit against the drop-in (which runs the search itself)."""
    from fastqsl_gb300 import api, synthetic as S
    rng = np.random.default_rng(sum(shape))
    ext = (12.0, 10.0, 10.0)
    lo = (-6.0, -5.0, 0.0)
    coords = []
    for n, e, a in zip(shape, ext, lo):
        w = rng.uniform(0.3, 3.0, n - 1)
        coords.append((a + np.concatenate([[0.0], np.cumsum(w)]) * (e / w.sum())).astype(np.float32))
    spec = S.bipole4_stretch(11, shape)
    Bx, By, Bz = S.make_field_coords(spec, *coords)
    m = 600
    pts = [rng.uniform(c[0], c[-1], m).astype(np.float32) for c in coords]
    # a third of the seeds on node coordinates (interval ends of the search)
    for d in range(3):
        pts[d][: m // 3] = rng.choice(coords[d], m // 3)
    xs, ys, zs = pts
    got_d = run_dropin_stretch(Bx, By, Bz, coords, False, xs, ys, zs, 0.01, 1.0, arith="fast")
    prm = P.reference_stretch(arith=P.ARITH_FAST)
    out = api.trace_stretch(*[torch.from_numpy(np.asfortranarray(b)) for b in (Bx, By, Bz)],
                            [torch.from_numpy(c).cuda() for c in coords], _dev(xs), _dev(ys), _dev(zs), prm,
                            s_len=0.01, uni=False)
    torch.cuda.synchronize()
    got_n = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    for k in F32 + I32 + ["LineLen"]:
        a, b = got_n[k], got_d[k]
        assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)]), k
