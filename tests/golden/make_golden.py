"""Generates the golden fixtures in tests/golden/ from the REFERENCE itself.

Run where the reference checkout exists ($QSL_REFERENCE_ROOT, default: a
directory named `reference` beside this repository):

    python oracle/build.py            # builds oracle/_ref from the reference sources
    python tests/golden/make_golden.py

What runs:
* tracing — the reference's own kernels (fastqslpy/cu/TraceBline.cu,
  TraceBlineAdaptive.cu, TraceBlineScott.cu, TraceBlineAdaptiveStretch.cu),
  compiled for the host by
  oracle/build_ref.sh (unmodified sources, -ffp-contract=off, except one
  line of TraceBlineScott.cu in a copy: its uninitialised tolerance set to
  TOL*tol_coef);
* Q assembly — the reference's own fastqslpy/FastQSL.py (QCalcPlane,
  CookPseudoLine, ResReshape) imported with NumPy standing in for CuPy, and
  the pseudo-line Q cells of demo/Q_RKF45CuPy.ipynb (cells 9-11) executed
  from the notebook file with the same substitution;
* field-line polylines — the reference's own fastqslpy/MagTool.py, with the
  np.int alias it needs restored (``make_golden.py magtool`` alone).

Inputs are the seeded synthetic fields of fastqsl_gb300.synthetic (the
reference's demo fields are not distributed); each fixture stores the field
spec and a fingerprint of the sampled field so the tests can regenerate it.
"""
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fastqsl_gb300 import synthetic as S  # noqa: E402

REF = os.environ.get("QSL_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))


def reference_fastqsl():
    """Imports the reference's fastqslpy/FastQSL.py with numpy as cupy."""
    sys.modules.setdefault("cupy", np)
    spec = importlib.util.spec_from_file_location("ref_FastQSL", os.path.join(REF, "fastqslpy", "FastQSL.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def notebook_cells(path, idx):
    with open(path) as f:
        nb = json.load(f)
    return ["".join(nb["cells"][i]["source"]) for i in idx]


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def trace_case(name, kind, spec_fn, seed, seeds_xy, z, s_len, tol_coef, twist=False):
    spec = spec_fn(seed)
    Bx, By, Bz = S.make_field(spec)
    (xr, yr, nx, ny) = seeds_xy
    xs, ys, zs, shp = S.plane_seeds(xr, yr, nx, ny, z)
    cur = (By * np.float32(0.3) + Bz, Bz - Bx, Bx * np.float32(0.5) + By) if twist else None
    out = oracle.trace_all("ref_" + kind, Bx, By, Bz, xs, ys, zs, s_len=s_len, tol_coef=tol_coef, curB=cur)
    meta = dict(kind=kind, spec=spec_fn.__name__, seed=seed, s_len=s_len, tol_coef=tol_coef, twist=twist,
                z=z, seeds=[list(xr), list(yr), nx, ny], fingerprint=S.field_fingerprint(Bx, By, Bz))
    save(name, meta=json.dumps(meta), inp_x=xs, inp_y=ys, inp_z=zs, **out)


def stretch_case(name, seed, z_ratio, uni, twist=False, s_len=0.01, tol_coef=1.0):
    """TraceAllBline of TraceBlineAdaptiveStretch.cu on bipole4_stretch over
    stretched_axes(z_ratio); 40 x 32 seeds at z = 1e-3 (as the reference's
    stretched notebook seeds just above the bottom face)."""
    spec = S.bipole4_stretch(seed)
    xa, ya, za = S.stretched_axes(spec.shape, z_ratio=z_ratio)
    Bx, By, Bz = S.make_field_coords(spec, xa, ya, za)
    xs, ys, zs, shp = S.plane_seeds((-5, 5), (-4, 4), 40, 32, 1e-3)
    cur = (By * np.float32(0.3) + Bz, Bz - Bx, Bx * np.float32(0.5) + By) if twist else None
    out = oracle.trace_all("ref_stretch", Bx, By, Bz, xs, ys, zs, s_len=s_len, tol_coef=tol_coef, curB=cur,
                           coords=(xa, ya, za), uni=uni)
    meta = dict(kind="stretch", spec="bipole4_stretch", seed=seed, z_ratio=z_ratio, uni=uni, s_len=s_len,
                tol_coef=tol_coef, twist=twist, fingerprint=S.field_fingerprint(Bx, By, Bz))
    save(name, meta=json.dumps(meta), inp_x=xs, inp_y=ys, inp_z=zs, xa=xa, ya=ya, za=za, **out)


def scott_case(name, seed, twist):
    """Whole-line TraceBlineScott (TraceBlineScott.cu:334-519) of the
    reference, built from the copy with its tolerance initialised
    (oracle/build_ref.sh), on bipole4_64: 40 x 36 seeds, all on z = 0
    without the twist (the reference's second direction is defined there:
    one direction of a bottom-plane seed is skipped), and with the twist
    every third seed at z = 6.5 and one below z = 0 (with the twist on every
    quantity the routine reads is set)."""
    spec = S.bipole4_64(seed)
    Bx, By, Bz = S.make_field(spec)
    xs, ys, zs, shp = S.plane_seeds((2, 61), (2, 61), 40, 36, 0.0)
    if twist:
        zs[::3] = 6.5
        zs[5] = -1.0
    cur = (By * np.float32(0.3) + Bz, Bz - Bx, Bx * np.float32(0.5) + By) if twist else None
    out = oracle.scott_all("ref_scott", Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0, curB=cur)
    meta = dict(kind="scott", spec="bipole4_64", seed=seed, s_len=0.25, tol_coef=1.0, twist=twist,
                fingerprint=S.field_fingerprint(Bx, By, Bz))
    save(name, meta=json.dumps(meta), inp_x=xs, inp_y=ys, inp_z=zs, **out)


def scott_cases():
    scott_case("scott_bipole4_64.npz", 2, False)
    scott_case("scott_twist_bipole4_64.npz", 1, True)


def curl_case():
    """curl_of_B_grid of the reference's FastQSL.py (NumPy as CuPy) on a
    small stretched grid."""
    FastQSL = reference_fastqsl()
    spec = S.bipole4_stretch(6, shape=(20, 16, 12))
    xa, ya, za = S.stretched_axes(spec.shape, z_ratio=1.08)
    Bx, By, Bz = S.make_field_coords(spec, xa, ya, za)
    cx, cy, cz = FastQSL.curl_of_B_grid(Bx, By, Bz, xa, ya, za)
    meta = dict(spec="bipole4_stretch", seed=6, shape=[20, 16, 12], z_ratio=1.08,
                fingerprint=S.field_fingerprint(Bx, By, Bz))
    save("curl_stretch.npz", meta=json.dumps(meta), xa=xa, ya=ya, za=za, curl_x=np.asarray(cx),
         curl_y=np.asarray(cy), curl_z=np.asarray(cz))


def probes_case():
    spec = S.bipole4_64(3)
    Bx, By, Bz = S.make_field(spec)
    rng = np.random.default_rng(7)
    m = 400
    pts = rng.uniform(-2.5, 65.5, size=(m, 3)).astype(np.float32)
    # include exact grid nodes, faces and cell edges
    pts[:40] = rng.integers(0, 64, size=(40, 3)).astype(np.float32)
    pts[40:60, 0] = 0.0
    pts[60:80, 1] = 63.0
    hs = rng.uniform(-2.0, 2.0, size=m).astype(np.float32)
    dims = rng.integers(0, 3, size=m).astype(np.int32)
    v9 = np.concatenate([pts, rng.normal(size=(m, 6)).astype(np.float32)], axis=1)
    pr = oracle.Probe("ref_rkf45", Bx, By, Bz)
    pr4 = oracle.Probe("ref_rk4", Bx, By, Bz)
    ps = oracle.Probe("ref_scott", Bx, By, Bz)
    res = dict(
        interp_unit=np.stack([pr.interp(p, True) for p in pts]),
        interp_raw=np.stack([pr.interp(p, False) for p in pts]),
        interp_scalar=np.array([[pr.interp_scalar(c, p) for c in range(3)] for p in pts], np.float32),
        checkflag=np.array([pr.checkflag(p) for p in pts], np.int32),
        rk4=np.stack([pr4.rk4(p, h) for p, h in zip(pts, hs)]),
        rkf45=np.stack([pr.rkf45(p, h) for p, h in zip(pts, hs)]),
        rk4_boundary=np.stack([pr.rk4_boundary(p, h, int(d)) for p, h, d in zip(pts, hs, dims)]),
        grad_unit_b=np.stack([ps.grad_unit_b(p) for p in pts]),
        f_scott=np.stack([ps.f_scott(v) for v in v9]),
    )
    sc = [ps.rkf45_scott(v, h) for v, h in zip(v9, hs)]
    res["rkf45_scott"] = np.stack([s[0] for s in sc])
    res["rkf45_scott_err"] = np.array([s[1] for s in sc], np.float32)
    meta = dict(spec="bipole4_64", seed=3, fingerprint=S.field_fingerprint(Bx, By, Bz))
    save("probes_bipole4_64.npz", meta=json.dumps(meta), pts=pts, hs=hs, dims=dims, v9=v9, **res)


def qmap_case():
    """The 2-D Q-map workflow of demo/Q_RKF45CuPy.ipynb (cells 6-11) on the
    64^3 four-charge field: main trace, QCalcPlane, CookPseudoLine,
    pseudo-line trace at tol_coef*0.1, Qcut and the merge."""
    FastQSL = reference_fastqsl()
    spec = S.bipole4_64(0)
    Bx, By, Bz = S.make_field(spec)
    interp_ratio = 2
    stride_step = 1 / interp_ratio
    x_range = [6, 56]
    y_range = [8, 50]
    nx = int(np.uint(interp_ratio * (x_range[1] - x_range[0])))
    ny = int(np.uint(interp_ratio * (y_range[1] - y_range[0])))
    xs, ys, zs, xy_shape = S.plane_seeds(x_range, y_range, nx, ny, 0.0001)
    tol_coef = 1.0
    s_len = 1.0 / 8.0
    o = oracle.trace_all("ref_rkf45", Bx, By, Bz, xs, ys, zs, s_len=s_len, tol_coef=tol_coef * 0.5)
    (x_end_arr, y_end_arr, z_end_arr, flag_end_arr,
     x_start_arr, y_start_arr, z_start_arr, flag_start_arr,
     Bx_in_arr, By_in_arr, Bz_in_arr,
     Bx_out_arr, By_out_arr, Bz_out_arr,
     Bx_0_arr, By_0_arr, Bz_0_arr, B_flag_arr) = FastQSL.ResReshape(
        xy_shape, o["end_x"], o["end_y"], o["end_z"], o["flag_end"],
        o["start_x"], o["start_y"], o["start_z"], o["flag_start"],
        o["B_start_x"], o["B_start_y"], o["B_start_z"], o["B_end_x"], o["B_end_y"], o["B_end_z"],
        o["B_this_x"], o["B_this_y"], o["B_this_z"], o["B_flag"])
    Q = FastQSL.QCalcPlane(x_end_arr, y_end_arr, z_end_arr, flag_end_arr,
                           x_start_arr, y_start_arr, z_start_arr, flag_start_arr,
                           Bx_in_arr, By_in_arr, Bz_in_arr, Bx_out_arr, By_out_arr, Bz_out_arr,
                           Bx_0_arr, By_0_arr, Bz_0_arr, B_flag_arr, stride_step)
    stride_this = np.float32(1.0 / interp_ratio)
    cook = FastQSL.CookPseudoLine(x_end_arr, y_end_arr, z_end_arr, flag_end_arr,
                                  x_start_arr, y_start_arr, z_start_arr, flag_start_arr,
                                  Bx_in_arr, By_in_arr, Bz_in_arr, Bx_out_arr, By_out_arr, Bz_out_arr,
                                  Bz_0_arr, B_flag_arr, stride_this)
    (cut_inp_x, cut_inp_y, cut_inp_z, cut_start_x, cut_start_y, cut_start_z, flag_cut_start,
     cut_end_x, cut_end_y, cut_end_z, flag_cut_end, Bx_inp_cut, By_inp_cut, Bz_inp_cut, B_flag_cut,
     Bx_start_cut, By_start_cut, Bz_start_cut, Bx_end_cut, By_end_cut, Bz_end_cut,
     N_cut, line_len_cut, Bz0_start, Bz0_end) = cook
    # cell 9: second trace on the pseudo seeds (tol_coef*0.1)
    o2 = oracle.trace_all("ref_rkf45", Bx, By, Bz, cut_inp_x, cut_inp_y, cut_inp_z, s_len=s_len,
                          tol_coef=np.float32(tol_coef * 0.1))
    cut_start_x, cut_start_y, cut_start_z = o2["start_x"], o2["start_y"], o2["start_z"]
    cut_end_x, cut_end_y, cut_end_z = o2["end_x"], o2["end_y"], o2["end_z"]
    flag_cut_start, flag_cut_end = o2["flag_start"], o2["flag_end"]
    # cells 10-11 of the notebook, run from the notebook file itself
    ns = dict(cupy=np, np=np, cut_inp_x=cut_inp_x, cut_start_x=cut_start_x, cut_start_y=cut_start_y,
              cut_start_z=cut_start_z, cut_end_x=cut_end_x, cut_end_y=cut_end_y, cut_end_z=cut_end_z,
              flag_cut_start=flag_cut_start, flag_cut_end=flag_cut_end, Bz0_end=Bz0_end, Bz0_start=Bz0_start,
              stride_this=stride_this, Q=Q, x_end_arr=x_end_arr, B_flag_arr=B_flag_arr)
    src10, src11 = notebook_cells(os.path.join(REF, "demo", "Q_RKF45CuPy.ipynb"), [10, 11])
    src10 = src10.replace("cupy.cuda.stream.get_current_stream().synchronize()", "")
    with np.errstate(all="ignore"):
        exec(compile(src10, "Q_RKF45CuPy.ipynb:cell10", "exec"), ns)
        exec(compile(src11, "Q_RKF45CuPy.ipynb:cell11", "exec"), ns)
    meta = dict(spec="bipole4_64", seed=0, x_range=x_range, y_range=y_range, interp_ratio=interp_ratio,
                s_len=s_len, tol_coef=tol_coef, fingerprint=S.field_fingerprint(Bx, By, Bz),
                xy_shape=list(xy_shape))
    save("qmap_rkf45_bipole4_64.npz", meta=json.dumps(meta),
         inp_x=xs, inp_y=ys, inp_z=zs,
         **{"main_" + k: v for k, v in o.items()},
         Q=Q, cut_inp_x=cut_inp_x, cut_inp_y=cut_inp_y, cut_inp_z=cut_inp_z,
         Bz0_start=Bz0_start, Bz0_end=Bz0_end, N_cut=np.asarray(N_cut),
         **{"cut_" + k: v for k, v in o2.items()},
         Qcut=ns["Qcut"], Q_all=ns["Q_all"], Q_final=ns["Q_final"])


def reference_magtool():
    """Imports the reference's fastqslpy/MagTool.py.  It calls np.int, which
    NumPy 1.24 removed; the builtin int it aliased is put back first."""
    if not hasattr(np, "int"):
        np.int = int
    spec = importlib.util.spec_from_file_location("ref_MagTool", os.path.join(REF, "fastqslpy", "MagTool.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MAGTOOL_SHAPE = (40, 32, 24)


def magtool_case():
    """fastqslpy/MagTool.py: TraceBline polylines (maxstep 800) from float32
    seeds on a 40 x 32 x 24 field (lines that rise above z = 24 run on along
    the clamped top plane until z > 40, the first axis length), and trilerp /
    Bnorm at float64 points inside, on and outside the box."""
    mt = reference_magtool()
    spec = S.charges_random(5, MAGTOOL_SHAPE, 5, depth=(2.0, 6.0))
    Bx, By, Bz = S.make_field(spec)
    rng = np.random.default_rng(17)
    seeds = np.stack([rng.uniform(2, 37, 7), rng.uniform(2, 29, 7), rng.uniform(0.5, 20, 7)], 1).astype(np.float32)
    seeds = np.concatenate([seeds, np.array([[39.6, 31.4, 23.7], [0.0, 0.0, 0.0]], np.float32)])
    lines = []
    for p in seeds:
        lx, ly, lz = mt.TraceBline(Bx, By, Bz, p.copy(), dr=0.25, maxstep=800)
        lines.append(np.stack([lx, ly, lz]))
    pts = np.concatenate([rng.uniform(-2, 42, (40, 3)),
                          np.array([[39.5, 31.5, 23.5], [40.0 - 1e-9, 0.3, 0.2], [-0.1, 31.99, 23.999],
                                    [12.0, 7.0, 3.0], [38.0, 30.5, 22.5]])])
    tri = np.stack([mt.trilerp(Bx, By, Bz, p.copy()) for p in pts])
    bn = np.stack([mt.Bnorm(Bx, By, Bz, p.copy()) for p in pts])
    save("magtool_charges5.npz", seed=np.int64(5), shape=np.array(MAGTOOL_SHAPE), seeds=seeds,
         lines=np.stack(lines), pts=pts, trilerp=tri, bnorm=bn,
         fingerprint=np.array([float(np.sum(Bx, dtype=np.float64)), float(np.sum(Bz, dtype=np.float64))]))


def main():
    if sys.argv[1:] == ["magtool"]:
        return magtool_case()
    if not oracle.ref_available("rkf45"):
        raise SystemExit("oracle/_ref not built: run python oracle/build.py in a checkout with the reference")
    if sys.argv[1:] == ["stretch"]:  # only the stretched-grid fixtures
        return stretch_cases()
    if sys.argv[1:] == ["curl"]:
        return curl_case()
    if sys.argv[1:] == ["scott"]:
        return scott_cases()
    trace_case("trace_rk4_bipole4_64.npz", "rk4", S.bipole4_64, 0, ((0, 63), (0, 63), 64, 64), 0.0, 0.1, 1.0)
    trace_case("trace_rkf45_bipole4_64.npz", "rkf45", S.bipole4_64, 0, ((0, 63), (0, 63), 64, 64), 1e-4,
               0.125, 0.5)
    trace_case("trace_rkf45_twist_bipole4_64.npz", "rkf45", S.bipole4_64, 1, ((2, 61), (2, 61), 40, 40), 1e-4,
               0.125, 1.0, twist=True)
    trace_case("trace_rk4_twist_bipole4_64.npz", "rk4", S.bipole4_64, 1, ((2, 61), (2, 61), 40, 40), 0.0,
               0.1, 1.0, twist=True)
    probes_case()
    scott_cases()
    qmap_case()
    stretch_cases()
    curl_case()
    magtool_case()


def stretch_cases():
    stretch_case("trace_stretch_bipole4s.npz", 1, 1.06, False)
    stretch_case("trace_stretch_uni_twist_bipole4s.npz", 2, 1.0, True, twist=True)


if __name__ == "__main__":
    main()
