"""Loading of the golden fixtures in tests/golden (made from the reference by
tests/golden/make_golden.py)."""
import json
import os

import numpy as np

from fastqsl_gb300 import synthetic as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SPECS = {"bipole4_64": S.bipole4_64}


def load(name):
    g = np.load(os.path.join(GOLDEN, name))
    meta = json.loads(str(g["meta"]))
    return g, meta


def field_for(meta):
    spec = SPECS[meta["spec"]](meta["seed"])
    Bx, By, Bz = S.make_field(spec)
    assert S.field_fingerprint(Bx, By, Bz) == meta["fingerprint"], "synthetic field differs from the fixture's"
    return Bx, By, Bz


def stretch_field_for(meta):
    """Field and node coordinates of a stretched-grid fixture."""
    spec = S.bipole4_stretch(meta["seed"])
    xa, ya, za = S.stretched_axes(spec.shape, z_ratio=meta["z_ratio"])
    Bx, By, Bz = S.make_field_coords(spec, xa, ya, za)
    assert S.field_fingerprint(Bx, By, Bz) == meta["fingerprint"], "synthetic field differs from the fixture's"
    return Bx, By, Bz, (xa, ya, za)


STRETCH_CASES = ["trace_stretch_bipole4s.npz", "trace_stretch_uni_twist_bipole4s.npz"]


def twist_current(Bx, By, Bz):
    """The stand-in current density the twist fixtures were made with."""
    return (By * np.float32(0.3) + Bz, Bz - Bx, Bx * np.float32(0.5) + By)


TRACE_CASES = {
    "trace_rk4_bipole4_64.npz": ("rk4", False),
    "trace_rkf45_bipole4_64.npz": ("rkf45", False),
    "trace_rkf45_twist_bipole4_64.npz": ("rkf45", True),
    "trace_rk4_twist_bipole4_64.npz": ("rk4", True),
}

FOOT_KEYS = ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z",
             "B_start_x", "B_start_y", "B_start_z", "B_end_x", "B_end_y", "B_end_z"]


def limit_mask(g):
    """Seeds whose both directions left the box (flag != 0); the reference's
    footpoint of a direction stopped by a limit is stale scratch memory."""
    return (g["flag_start"] != 0) & (g["flag_end"] != 0)


def magtool_case(name="magtool_charges5.npz"):
    """The MagTool fixture and its field (charges_random(seed, shape, 5,
    depth 2-6), float32 (nx, ny, nz) Fortran order); checks the fingerprint."""
    g = np.load(os.path.join(GOLDEN, name))
    spec = S.charges_random(int(g["seed"]), tuple(int(v) for v in g["shape"]), 5, depth=(2.0, 6.0))
    B = S.make_field(spec)
    fp = [float(np.sum(B[0], dtype=np.float64)), float(np.sum(B[2], dtype=np.float64))]
    assert np.allclose(fp, g["fingerprint"], rtol=0, atol=1e-9 * max(1.0, abs(fp[0]))), "field generator changed"
    return g, B
