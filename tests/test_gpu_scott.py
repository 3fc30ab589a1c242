"""GPU Scott deviation-vector tracer (reference: fastqslpy/cu/
TraceBlineScott.cu:334-595).

* drop-in TraceAllBlineScott (exact arithmetic, central differences) against
  the reference's own whole-line routine (golden fixtures from the reference
  built with its uninitialised tolerance set to TOL*tol_coef, the one line
  the build changes): identical exit faces on >= 99.9 % of the seeds the
  reference defines, footpoints within 1e-3 cell and q_0 / q_perp within
  1e-3 relative on >= 99.5 % of the lines (the reference's host powf rounds
  differently from the correctly rounded power of the exact kernels in
  ~6e-4 of calls, which moves a few steps);
* the same drop-in against the oracle restatement with the same correctly
  rounded power: identical flags, footpoints within 1e-3 cell on >= 99.5 %,
  q_perp within 1e-3 relative on >= 99 %;
* fast arithmetic, both gradients, fp16 bricks included: flags >= 99 %;
  log10 q_perp within 1e-2 of the FP64 oracle (median); with a current
  density, the twist no further from the FP64 oracle than the reference's
  own FP32 rounding is (within a factor 1.5, median and 90th percentile).
"""
import numpy as np
import pytest
import torch

from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu


def _case():
    from fastqsl_gb300 import synthetic as S
    spec = S.charges_random(8, (48, 44, 36), 6)
    Bx, By, Bz = S.make_field(spec)
    xs, ys, zs, _ = S.plane_seeds((2, 45), (2, 41), 40, 36, 0.0)
    zs[::3] = 6.5  # some seeds above the bottom plane
    zs[5] = -1.0   # a skipped seed (below z = 0)
    return Bx, By, Bz, xs, ys, zs


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def run_dropin_scott(Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0, curB=None):
    """TraceAllBlineScott through the drop-in (C ABI), the reference's
    30-argument order; returns numpy outputs keyed like the oracle's."""
    from fastqsl_gb300.api import as_xfast
    from fastqsl_gb300.fastqslpy import kernels
    n = xs.size
    b = [as_xfast(torch.from_numpy(np.asfortranarray(a))) for a in (Bx, By, Bz)]
    f = {k: torch.zeros(n, dtype=torch.float32, device="cuda") for k in
         ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z", "B_this_x", "B_this_y", "B_this_z", "q_0",
          "q_perp"]}
    fl = {k: torch.zeros(n, dtype=torch.int32, device="cuda") for k in ("flag_start", "flag_end")}
    ll = torch.zeros(n, dtype=torch.float64, device="cuda")
    tw = torch.zeros(n, dtype=torch.float64, device="cuda")
    dummy = torch.zeros((1, 1), dtype=torch.float32, device="cuda")
    if curB is not None:
        c = [as_xfast(torch.from_numpy(np.asfortranarray(a))) for a in curB]
        flag = torch.tensor([True], device="cuda")
    else:
        c = [dummy] * 3
        flag = torch.tensor([False], device="cuda")
    k = kernels.compileTraceBlineScott()
    k((128, 1, 1), (28, 1), (b[0], b[1], b[2], torch.tensor(list(Bx.shape), dtype=torch.int32, device="cuda"),
                             c[0], c[1], c[2], tw, flag,
                             _dev(xs), _dev(ys), _dev(zs), torch.tensor([0, 0, 1.0], device="cuda"),
                             f["start_x"], f["start_y"], f["start_z"], fl["flag_start"], f["end_x"], f["end_y"],
                             f["end_z"], fl["flag_end"], f["B_this_x"], f["B_this_y"], f["B_this_z"], f["q_0"],
                             f["q_perp"], torch.tensor([s_len], device="cuda"),
                             torch.tensor([n], dtype=torch.int64, device="cuda"), ll,
                             torch.tensor([tol_coef], device="cuda")))
    torch.cuda.synchronize()
    out = {kk: v.cpu().numpy() for kk, v in {**f, **fl}.items()}
    out["LineLen"] = ll.cpu().numpy()
    out["twist"] = tw.cpu().numpy()
    return out


@pytest.mark.parametrize("name", ["scott_bipole4_64.npz", "scott_twist_bipole4_64.npz"])
def test_dropin_scott_exact_matches_reference(cuda, name):
    """Whole lines against the reference's own TraceBlineScott."""
    import golden_util as G
    g, meta = G.load(name)
    Bx, By, Bz = G.field_for(meta)
    cur = G.twist_current(Bx, By, Bz) if meta["twist"] else None
    got = run_dropin_scott(Bx, By, Bz, g["inp_x"], g["inp_y"], g["inp_z"], meta["s_len"], meta["tol_coef"], cur)
    defined = g["inp_z"] >= 0
    same = (got["flag_start"] == g["flag_start"]) & (got["flag_end"] == g["flag_end"])
    assert same[defined].mean() >= 0.999, same[defined].mean()
    np.testing.assert_array_equal(got["B_this_x"][defined], g["B_this_x"][defined])
    live = G.scott_live(g) & same
    assert live.mean() > 0.85
    d = np.zeros(len(live))
    for a, b in (("start_x", "end_x"), ("start_y", "end_y"), ("start_z", "end_z")):
        d = np.maximum(d, np.maximum(np.abs(got[a] - g[a]), np.abs(got[b] - g[b])))
    assert (d[live] <= 1e-3).mean() >= 0.995, (d[live] <= 1e-3).mean()
    for k in ("q_0", "q_perp"):
        ok = live & (g[k] > 0)
        rel = np.abs(got[k][ok] - g[k][ok]) / g[k][ok]
        assert (rel <= 1e-3).mean() >= 0.995, (k, np.quantile(rel, [0.5, 0.99]))
    if meta["twist"]:
        rel = np.abs(got["twist"][live] - g["twist"][live]) / np.maximum(np.abs(g["twist"][live]), 1e-6)
        assert (rel <= 1e-3).mean() >= 0.995, np.quantile(rel, [0.5, 0.99])


def test_dropin_scott_exact_matches_oracle(cuda, oracle_port):
    Bx, By, Bz, xs, ys, zs = _case()
    ref = oracle_port.scott_all("port32cr", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0,
                                params=P.reference_scott())
    out = run_dropin_scott(Bx, By, Bz, xs, ys, zs)
    fl = [out["flag_start"], out["flag_end"]]
    got = {"end_x": out["end_x"], "start_y": out["start_y"], "qp": out["q_perp"]}
    np.testing.assert_array_equal(fl[0], ref["flag_start"])
    np.testing.assert_array_equal(fl[1], ref["flag_end"])
    np.testing.assert_array_equal(out["B_this_x"], ref["B_this_x"])
    live = (ref["flag_start"] != 0) & (ref["flag_end"] != 0)
    d = np.maximum(np.abs(got["end_x"] - ref["end_x"]), np.abs(got["start_y"] - ref["start_y"]))
    assert (d[live] <= 1e-3).mean() >= 0.995
    qp, qr = got["qp"], ref["q_perp"]
    ok = live & (qr > 0)
    rel = np.abs(qp[ok] - qr[ok]) / qr[ok]
    assert (rel <= 1e-3).mean() >= 0.99, np.quantile(rel, [0.5, 0.99])


@pytest.mark.parametrize("layout,grad", [("soa", "fd"), ("soa", "analytic"), ("h4b", "analytic"), ("h8c", "analytic"),
                                         ("h8c", "fd")])
def test_fast_scott_vs_fp64_oracle(cuda, oracle_port, layout, grad):
    from fastqsl_gb300 import api
    Bx, By, Bz, xs, ys, zs = _case()
    prm = P.reference_scott(arith=P.ARITH_FAST)
    prm.tol = 1e-5
    prm.h_min = 1e-3
    prm.h_max = 1.0
    ref = oracle_port.scott_all("port64", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0,
                                params=prm.copy(arith=P.ARITH_EXACT))
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout=layout)
    out = api.trace_scott(fs, _dev(xs), _dev(ys), _dev(zs), prm, s_len=0.25, grad=grad)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    flags = ((got["flag_start"] == ref["flag_start"]) & (got["flag_end"] == ref["flag_end"])).mean()
    assert flags >= 0.99, flags
    ok = (ref["q_perp"] > 0) & (got["q_perp"] > 0) & (got["flag_end"] == ref["flag_end"]) & \
         (got["flag_start"] == ref["flag_start"]) & (ref["flag_start"] != 0) & (ref["flag_end"] != 0)
    d = np.abs(np.log10(got["q_perp"][ok]) - np.log10(ref["q_perp"][ok]))
    assert np.median(d) <= 1e-2, np.median(d)


@pytest.mark.parametrize("layout,grad", [("soa", "fd"), ("h4b", "analytic")])
def test_fast_scott_twist_vs_fp64_oracle(cuda, oracle_port, layout, grad):
    """The twist integral of the fast Scott tracer (the main tracer's fast
    integrand and 1 / (4 pi) product per step) against the FP64 oracle, on
    lines whose exit faces agree, measured against the reference's own FP32
    rounding (the oracle restatement pinned to it, port32cr): on these Scott
    lines the reference's FP32 twist is itself 7-17 % (median) off FP64 (the
    line lengths move with the step sequence), so the fast kernel must be
    no further off than that, within a factor 1.5."""
    import golden_util as G
    from fastqsl_gb300 import api
    Bx, By, Bz, xs, ys, zs = _case()
    cur = G.twist_current(Bx, By, Bz)
    prm = P.reference_scott(arith=P.ARITH_FAST)
    prm.tol = 1e-5
    prm.h_min = 1e-3
    prm.h_max = 1.0
    ex = prm.copy(arith=P.ARITH_EXACT)
    ref = oracle_port.scott_all("port64", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0, params=ex, curB=cur)
    r32 = oracle_port.scott_all("port32cr", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0, params=ex, curB=cur)
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout=layout)
    curd = [api.as_xfast(torch.from_numpy(np.asfortranarray(c))) for c in cur]  # x-fastest, as the field
    out = api.trace_scott(fs, _dev(xs), _dev(ys), _dev(zs), prm, s_len=0.25, grad=grad, curB=curd)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items() if v is not None}

    def err(o):
        # seeds on the bottom plane trace one direction (flag_start 0, as
        # the reference); lines whose flags agree and which carry a twist
        same = (o["flag_start"] == ref["flag_start"]) & (o["flag_end"] == ref["flag_end"]) & (np.abs(ref["twist"]) > 0)
        rel = np.abs(o["twist"][same] - ref["twist"][same]) / np.maximum(np.abs(ref["twist"][same]), 1e-3)
        return same.mean(), np.median(rel), np.quantile(rel, 0.9)

    lines, med, p90 = err(got)
    _, med32, p90_32 = err(r32)
    print(layout, grad, "scott twist lines %.3f rel err median %.2e p90 %.2e (reference FP32: %.2e / %.2e)" % (
        lines, med, p90, med32, p90_32))
    assert lines > 0.5
    assert med <= 1.5 * med32 and p90 <= 1.5 * p90_32, (med, p90, med32, p90_32)
