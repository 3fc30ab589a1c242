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

# whole-line TraceBlineScott fixtures: name -> twist on
SCOTT_CASES = {"scott_bipole4_64.npz": False, "scott_twist_bipole4_64.npz": True}


def scott_live(g):
    """Seeds whose two directions both ended on a face (flags 1-6): the
    reference routine leaves its footpoints and q unset on a line stopped by
    the shared step limit, ended on an edge (flag 42), or skipped (z < 0)."""
    fs, fe = g["flag_start"], g["flag_end"]
    return (fs >= 1) & (fs <= 6) & (fe >= 1) & (fe <= 6)


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


def fp16_exact_field(B, brick=8):
    """A field the fp16 stores hold exactly: every 8^3-cell brick's largest
    |component| (over its 9^3 nodes) raised to a power of two at that node,
    then every node rounded to 11 significant bits of the largest such scale
    among the bricks that hold it.  Dividing by a power-of-two scale and
    rounding to fp16 then changes no value, so the brick store (per-brick
    scale) and the cell-record store (per-cell power-of-two scale) see the
    float32 field's own node values, and a trace on them differs from one on
    the float32 field only by arithmetic."""
    B = [np.array(b, np.float64) for b in B]
    nx, ny, nz = B[0].shape
    sls = [(slice(i, min(i + brick + 1, nx)), slice(j, min(j + brick + 1, ny)), slice(k, min(k + brick + 1, nz)))
           for i in range(0, nx - 1, brick) for j in range(0, ny - 1, brick) for k in range(0, nz - 1, brick)]
    for _ in range(50):
        changed = 0
        for sl in sls:
            m = [np.abs(b[sl]).max() for b in B]
            c = int(np.argmax(m))
            if m[c] == 0:
                continue
            p = 2.0 ** np.ceil(np.log2(m[c]))
            if p != m[c]:
                blk = B[c][sl]
                idx = np.unravel_index(np.argmax(np.abs(blk)), blk.shape)
                blk[idx] = np.sign(blk[idx]) * p
                changed += 1
        if not changed:
            break
    E = np.full(B[0].shape, -200.0)
    for sl in sls:
        m = max(np.abs(b[sl]).max() for b in B)
        if m > 0:
            E[sl] = np.maximum(E[sl], np.log2(m))
    q = 2.0 ** (E - 11)
    return [np.asfortranarray((np.round(b / q) * q).astype(np.float32)) for b in B]
