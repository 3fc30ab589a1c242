"""Hybrid finite-difference + Scott Q on the GPU (QMapPlan(hybrid=True):
qsl_hybrid_select -> qsl_trace_scott on the selected seeds -> qsl_hybrid_merge)
against the FP64 oracle of the same workflow (oracle.qassembly.qmap_hybrid,
whose merge is pinned to demo/Q_RKF45MixCuPyDiffScott.ipynb cell 9)."""
import numpy as np
import pytest
import torch

from fastqsl_gb300 import params as P

pytestmark = pytest.mark.gpu


def test_hybrid_qmap_vs_fp64_oracle(cuda, oracle_port):
    from fastqsl_gb300 import api, synthetic as S
    from oracle import qassembly as QA
    spec = S.charges_random(21, (80, 72, 48), 6)
    Bx, By, Bz = S.make_field(spec)
    n0, n1 = 40, 48
    zs = [0.0, 6.0, 13.5]
    stride = 1.5
    xs, ys, zz = api.plane_seed_grid(4.0, 4.0 + stride * (n1 - 1), n1, 4.0, 4.0 + stride * (n0 - 1), n0, zs)
    prm = P.absolute_rkf45()
    fs = api.FieldStore(*[torch.from_numpy(b) for b in (Bx, By, Bz)], layout="soa")
    hyb = api.QMapPlan(n0, n1, len(zs), hybrid=True)
    Q = hyb.run(fs, xs, ys, zz, prm, s_len=0.25, stride=stride, scott_grad="fd").cpu().numpy()
    nsel = int(hyb.hcount.item())
    fd = api.QMapPlan(n0, n1, len(zs), pseudo=False)
    Qfd = fd.run(fs, xs, ys, zz, prm, s_len=0.25, stride=stride).cpu().numpy()
    # pixels the finite differences serve are untouched
    bf = hyb.main["B_flag"].cpu().numpy().reshape(len(zs), n0, n1)[:, 1:-1, 1:-1]
    sel = (bf != 0) | np.isnan(Qfd)
    assert sel.sum() == nsel and nsel > 0
    np.testing.assert_array_equal(Q[~sel], Qfd[~sel])
    # against the FP64 workflow
    prm64 = P.absolute_rkf45(arith=P.ARITH_EXACT)
    sc64 = P.reference_scott(arith=P.ARITH_EXACT).copy(tol=prm64.tol, h_min=prm64.h_min, h_max=prm64.h_max)
    tr = lambda a, b, c: oracle_port.trace_all("port64", Bx, By, Bz, a, b, c, s_len=0.25, params=prm64)  # noqa
    st = lambda a, b, c: oracle_port.scott_all("port64", Bx, By, Bz, a, b, c, s_len=0.25, params=sc64)  # noqa
    Qref, nref = QA.qmap_hybrid(tr, st, xs.cpu().numpy(), ys.cpu().numpy(), zz.cpu().numpy(), len(zs), n0, n1,
                                stride)
    assert abs(nref - nsel) <= max(3, 0.02 * nref)
    nan_same = np.isnan(Q) == np.isnan(Qref)
    assert nan_same.mean() >= 0.99
    # the Scott tracer leaves q_perp 0 where a line does not reach the box
    # faces at both ends; those pixels must agree too
    both = ~np.isnan(Q) & ~np.isnan(Qref)
    assert ((Q[both] == 0) == (Qref[both] == 0)).mean() >= 0.99
    ok = both & (Q > 0) & (Qref > 0)
    d = np.abs(np.log10(Q[ok]) - np.log10(Qref[ok]))
    assert np.median(d) <= 1e-3 and np.quantile(d, 0.99) <= 1e-2, (np.median(d), np.quantile(d, 0.99))
    ds = np.abs(np.log10(Q[ok & sel]) - np.log10(Qref[ok & sel]))
    assert np.median(ds) <= 1e-2, np.median(ds)
