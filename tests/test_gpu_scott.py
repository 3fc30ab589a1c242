"""GPU Scott deviation-vector tracer (reference: fastqslpy/cu/
TraceBlineScott.cu:334-595) against the oracle's restatement.

The reference kernel reads its tolerance uninitialised, so whole-line parity
is against the oracle (which fixes tol = 1e-3*tol_coef); the oracle's Scott
building blocks (gradient, right-hand side, one RKF45 step) are pinned bit
for bit to the reference in test_oracle_golden.py.
* drop-in TraceAllBlineScott (exact arithmetic, central differences) vs the
  oracle with the same correctly rounded power: identical flags, footpoints
  within 1e-3 cell on >= 99.5 %, q_perp within 1e-3 relative on >= 99 %;
* fast arithmetic, both gradients, fp16 bricks included: flags >= 99 %;
  log10 q_perp within 1e-2 of the FP64 oracle (median).
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


def test_dropin_scott_exact_matches_oracle(cuda, oracle_port):
    from fastqsl_gb300.api import as_xfast
    from fastqsl_gb300.fastqslpy import kernels
    Bx, By, Bz, xs, ys, zs = _case()
    ref = oracle_port.scott_all("port32cr", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0,
                                params=P.reference_scott())
    n = xs.size
    b = [as_xfast(torch.from_numpy(a)) for a in (Bx, By, Bz)]
    f = {k: torch.zeros(n, dtype=torch.float32, device="cuda") for k in
         ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z", "bx", "by", "bz", "q0", "qp"]}
    fl = [torch.zeros(n, dtype=torch.int32, device="cuda") for _ in range(2)]
    ll = torch.zeros(n, dtype=torch.float64, device="cuda")
    dummy = torch.zeros((1, 1), dtype=torch.float32, device="cuda")
    k = kernels.compileTraceBlineScott()
    k((128, 1, 1), (28, 1), (b[0], b[1], b[2], torch.tensor(list(Bx.shape), dtype=torch.int32, device="cuda"),
                             dummy, dummy, dummy, dummy, torch.tensor([False], device="cuda"),
                             _dev(xs), _dev(ys), _dev(zs), torch.tensor([0, 0, 1.0], device="cuda"),
                             f["start_x"], f["start_y"], f["start_z"], fl[0], f["end_x"], f["end_y"], f["end_z"],
                             fl[1], f["bx"], f["by"], f["bz"], f["q0"], f["qp"],
                             torch.tensor([0.25], device="cuda"), torch.tensor([n], dtype=torch.int64,
                                                                               device="cuda"), ll,
                             torch.tensor([1.0], device="cuda")))
    torch.cuda.synchronize()
    got = {kk: v.cpu().numpy() for kk, v in f.items()}
    np.testing.assert_array_equal(fl[0].cpu().numpy(), ref["flag_start"])
    np.testing.assert_array_equal(fl[1].cpu().numpy(), ref["flag_end"])
    np.testing.assert_array_equal(got["bx"], ref["B_this_x"])
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
