"""Seeded synthetic magnetic fields and seed grids for the benchmark and test
workloads.

The reference's demo fields (IDL ``.sav`` extrapolations of solar active
regions) are not distributed with it, so every workload here is a seeded
analytic field sampled on integer grid nodes:

* potential fields of sub-surface point charges, ``B = sum_i q_i (r - r_i) / |r - r_i|^3``;
* a uniformly twisted flux tube along x, ``B_x = B0 exp(-r^2/a^2)``,
  ``B_phi = T r B_x`` with ``T = 2 pi turns / L_x`` (divergence free because
  neither component depends on x or on the azimuth).

Fields are returned as three float32 arrays of shape ``(nx, ny, nz)`` with x
fastest in memory (Fortran order), the layout the reference kernels index
(``fastqslpy/cu/TraceBlineAdaptive.cu:36-39``).  The arithmetic uses only
+, -, *, / and sqrt in float64, so the same seed gives bit-identical fields on
any IEEE machine and on the GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field as dc_field

import numpy as np
import torch


@dataclass
class ChargeSet:
    pos: np.ndarray  # (m, 3) float64, grid coordinates
    q: np.ndarray    # (m,) float64


@dataclass
class Tube:
    y0: float
    z0: float
    radius: float
    b0: float
    turns: float


@dataclass
class FieldSpec:
    shape: tuple
    charges: ChargeSet | None = None
    tube: Tube | None = None
    name: str = ""
    meta: dict = dc_field(default_factory=dict)


def _zslab_field(spec: FieldSpec, z0: int, z1: int, device) -> tuple:
    nx, ny, nz = spec.shape
    f64 = torch.float64
    x = torch.arange(nx, dtype=f64, device=device).view(1, 1, nx)
    y = torch.arange(ny, dtype=f64, device=device).view(1, ny, 1)
    z = torch.arange(z0, z1, dtype=f64, device=device).view(z1 - z0, 1, 1)
    shp = (z1 - z0, ny, nx)
    bx = torch.zeros(shp, dtype=f64, device=device)
    by = torch.zeros(shp, dtype=f64, device=device)
    bz = torch.zeros(shp, dtype=f64, device=device)
    if spec.charges is not None:
        for (cx, cy, cz), q in zip(spec.charges.pos.tolist(), spec.charges.q.tolist()):
            dx = x - cx
            dy = y - cy
            dz = z - cz
            r2 = (dx * dx + dy * dy) + dz * dz
            inv = q / (r2 * torch.sqrt(r2))
            bx += dx * inv
            by += dy * inv
            bz += dz * inv
    if spec.tube is not None:
        t = spec.tube
        dy = y - t.y0
        dz = z - t.z0
        r2 = dy * dy + dz * dz
        # exp via torch on float64; identical across IEEE machines to within
        # libm rounding, which the float32 cast absorbs except at ties.
        ax = t.b0 * torch.exp(-r2 / (t.radius * t.radius))
        tw = 2.0 * math.pi * t.turns / nx
        bx += ax.expand(shp)
        by += (-tw * ax * dz).expand(shp)
        bz += (tw * ax * dy).expand(shp)
    return bx.float(), by.float(), bz.float()


def make_field(spec: FieldSpec, device="cpu", as_numpy=None, zchunk=None):
    """Samples the field on the grid.  Returns (Bx, By, Bz): torch tensors of
    shape (nx, ny, nz) with x fastest (strides (1, nx, nx*ny)) on `device`, or
    numpy Fortran-order arrays when `as_numpy` (default: device == 'cpu')."""
    nx, ny, nz = spec.shape
    if as_numpy is None:
        as_numpy = str(device) == "cpu"
    dev = torch.device(device)
    if zchunk is None:
        zchunk = max(1, min(nz, (1 << 24) // max(1, nx * ny)))
    out = [torch.empty((nz, ny, nx), dtype=torch.float32, device=dev) for _ in range(3)]
    for z0 in range(0, nz, zchunk):
        z1 = min(nz, z0 + zchunk)
        parts = _zslab_field(spec, z0, z1, dev)
        for o, p in zip(out, parts):
            o[z0:z1] = p
    # (nz, ny, nx) C-order == (nx, ny, nz) x-fastest
    res = [o.permute(2, 1, 0) for o in out]
    if as_numpy:
        return tuple(np.asfortranarray(r.cpu().numpy()) for r in res)
    return tuple(res)


# --------------------------------------------------------------------------
# Workloads (one per benchmark configuration)
# --------------------------------------------------------------------------

def bipole4_64(seed=0) -> FieldSpec:
    """64^3 field of 4 point charges at depth 8 below z = 0, (x, y) uniform in
    [0, 63]^2, strengths +-U(0.5, 1.5) shifted to net zero."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(0.0, 63.0, size=(4, 2))
    mag = rng.uniform(0.5, 1.5, size=4)
    sgn = rng.choice([-1.0, 1.0], size=4)
    q = mag * sgn
    q = q - q.mean()
    pos = np.column_stack([xy, np.full(4, -8.0)])
    return FieldSpec((64, 64, 64), ChargeSet(pos, q), None, "charges4-64c")


def bipole_tube_256(seed=0) -> FieldSpec:
    """256x256x128: charges +1/-1 at depth 10 under (96,128) and (160,128)
    plus a flux tube along x at (y, z) = (128, 40), radius 10, 1.5 turns over
    the box, B0 = 2e-3."""
    pos = np.array([[96.0, 128.0, -10.0], [160.0, 128.0, -10.0]])
    q = np.array([1.0, -1.0])
    return FieldSpec((256, 256, 128), ChargeSet(pos, q), Tube(128.0, 40.0, 10.0, 2e-3, 1.5),
                     "bipole+tube-256x256x128")


def charges32_512(seed=0, shape=(512, 512, 256), n=32) -> FieldSpec:
    """512x512x256 field of 32 charges at depth U(4, 20), (x, y) uniform over
    the box, strengths +-U(0.2, 2) (null points and separators appear)."""
    rng = np.random.default_rng(seed)
    nx, ny, _ = shape
    x = rng.uniform(0.0, nx - 1.0, size=n)
    y = rng.uniform(0.0, ny - 1.0, size=n)
    d = rng.uniform(4.0, 20.0, size=n)
    q = rng.uniform(0.2, 2.0, size=n) * rng.choice([-1.0, 1.0], size=n)
    pos = np.column_stack([x, y, -d])
    return FieldSpec(tuple(shape), ChargeSet(pos, q), None, f"charges{n}-{nx}x{ny}x{shape[2]}")


def charges_random(seed, shape, n_charges, depth=(4.0, 20.0), strength=(0.2, 2.0)) -> FieldSpec:
    rng = np.random.default_rng(seed)
    nx, ny, _ = shape
    x = rng.uniform(0.0, nx - 1.0, size=n_charges)
    y = rng.uniform(0.0, ny - 1.0, size=n_charges)
    d = rng.uniform(*depth, size=n_charges)
    q = rng.uniform(*strength, size=n_charges) * rng.choice([-1.0, 1.0], size=n_charges)
    return FieldSpec(tuple(shape), ChargeSet(np.column_stack([x, y, -d]), q), None,
                     f"charges{n_charges}-{'x'.join(map(str, shape))}")


def charges_tube(seed, shape, n_charges=8) -> FieldSpec:
    """Point charges plus a twisted tube along x with seeded height, radius,
    strength and twist (serving-stream fields)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    x = rng.uniform(0.0, nx - 1.0, size=n_charges)
    y = rng.uniform(0.0, ny - 1.0, size=n_charges)
    d = rng.uniform(4.0, 20.0, size=n_charges)
    q = rng.uniform(0.5, 1.5, size=n_charges) * rng.choice([-1.0, 1.0], size=n_charges)
    tube = Tube(float(rng.uniform(0.3, 0.7) * ny), float(rng.uniform(0.1, 0.3) * nz),
                float(rng.uniform(6.0, 14.0)), float(rng.uniform(1e-3, 4e-3)), float(rng.uniform(0.5, 2.0)))
    return FieldSpec(tuple(shape), ChargeSet(np.column_stack([x, y, -d]), q), tube,
                     f"charges{n_charges}+tube-{'x'.join(map(str, shape))}")


# --------------------------------------------------------------------------
# Stretched (non-uniform) grids
# --------------------------------------------------------------------------

def stretched_axes(shape, extent=(12.0, 10.0, 10.0), z_ratio=1.06):
    """Node coordinates of a stretched grid like the reference's stretched
    demo (TD7stretch1.sav: x, y uniform, z spacing growing with height):
    x and y uniform over [-extent/2, extent/2], z from 0 with spacing growing
    geometrically by z_ratio per cell, scaled to `extent[2]`.  float32."""
    nx, ny, nz = shape
    xa = np.linspace(-extent[0] / 2, extent[0] / 2, nx).astype(np.float32)
    ya = np.linspace(-extent[1] / 2, extent[1] / 2, ny).astype(np.float32)
    dz = z_ratio ** np.arange(nz - 1)
    za = np.concatenate([[0.0], np.cumsum(dz)])
    za = (za * (extent[2] / za[-1])).astype(np.float32)
    return xa, ya, za


def make_field_coords(spec: FieldSpec, xa, ya, za):
    """The field of `spec` (charges only) sampled at the nodes of a
    rectilinear grid with coordinates xa, ya, za; (nx, ny, nz) float32
    Fortran-order arrays, the same float64 arithmetic as make_field."""
    x = np.asarray(xa, np.float64).reshape(-1, 1, 1)
    y = np.asarray(ya, np.float64).reshape(1, -1, 1)
    z = np.asarray(za, np.float64).reshape(1, 1, -1)
    shp = (x.shape[0], y.shape[1], z.shape[2])
    bx = np.zeros(shp)
    by = np.zeros(shp)
    bz = np.zeros(shp)
    for (cx, cy, cz), q in zip(spec.charges.pos.tolist(), spec.charges.q.tolist()):
        dx = x - cx
        dy = y - cy
        dz = z - cz
        r2 = (dx * dx + dy * dy) + dz * dz
        inv = q / (r2 * np.sqrt(r2))
        bx = bx + dx * inv
        by = by + dy * inv
        bz = bz + dz * inv
    return tuple(np.asfortranarray(a.astype(np.float32)) for a in (bx, by, bz))


def bipole4_stretch(seed=0, shape=(48, 40, 36)) -> FieldSpec:
    """4 charges at depth 0.8 below z = 0 of the stretched_axes box, (x, y)
    uniform in the central 80 %, strengths +-U(0.5, 1.5) shifted to net zero."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-0.4, 0.4, size=(4, 2)) * np.array([12.0, 10.0])
    mag = rng.uniform(0.5, 1.5, size=4)
    q = mag * rng.choice([-1.0, 1.0], size=4)
    q = q - q.mean()
    pos = np.column_stack([xy, np.full(4, -0.8)])
    return FieldSpec(tuple(shape), ChargeSet(pos, q), None, f"charges4-stretch-{'x'.join(map(str, shape))}")


def plane_seeds(x_range, y_range, nx, ny, z, indexing="xy"):
    """Seed grid on a z = const plane, built like the reference notebooks
    (``cupy.linspace`` per axis, ``meshgrid``, flattened).  Returns
    (x, y, z) float32 arrays and the 2-D shape."""
    xi = np.linspace(x_range[0], x_range[1], nx, dtype=np.float32)
    yi = np.linspace(y_range[0], y_range[1], ny, dtype=np.float32)
    xa, ya = np.meshgrid(xi, yi, indexing=indexing)
    shp = xa.shape
    xs = xa.ravel().astype(np.float32)
    ys = ya.ravel().astype(np.float32)
    zs = np.full_like(xs, np.float32(z))
    return xs, ys, zs, shp


def field_fingerprint(bx, by, bz) -> str:
    """Short hash of the three arrays' bytes in x-fastest order."""
    import hashlib
    h = hashlib.sha256()
    for a in (bx, by, bz):
        if isinstance(a, torch.Tensor):
            a = a.detach().cpu().numpy()
        h.update(np.ascontiguousarray(np.asarray(a).transpose(2, 1, 0)).tobytes())
    return h.hexdigest()[:16]


def cutting_plane(shape, normal, n0, n1, spacing=None, center=None):
    """Seeds on an arbitrarily oriented plane through `center` (default: box
    centre) with unit normal `normal`: an (n0, n1) grid along two in-plane
    axes u (columns) and v (rows), spacing chosen so the grid stays inside the
    box unless given.  Returns float32 (x, y, z) of the flattened grid, the
    normal (float32) and the spacing (the Q stride)."""
    nx, ny, nz = shape
    n = np.asarray(normal, np.float64)
    n = n / np.linalg.norm(n)
    e = np.eye(3)[int(np.argmin(np.abs(n)))]
    u = np.cross(n, e)
    u /= np.linalg.norm(u)
    v = np.cross(n, u)
    c = np.array([(nx - 1) / 2.0, (ny - 1) / 2.0, (nz - 1) / 2.0]) if center is None else np.asarray(center, float)
    if spacing is None:
        half = 0.45 * min(nx - 1, ny - 1, nz - 1)  # corners of the grid stay inside the box
        spacing = 2 * half / (max(n0, n1) - 1) / np.sqrt(2.0)
    a = (np.arange(n1) - (n1 - 1) / 2.0) * spacing
    b = (np.arange(n0) - (n0 - 1) / 2.0) * spacing
    B, A = np.meshgrid(b, a, indexing="ij")
    pts = c[None, None, :] + A[..., None] * u[None, None, :] + B[..., None] * v[None, None, :]
    pts = pts.reshape(-1, 3).astype(np.float32)
    return pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), n.astype(np.float32), float(spacing)
