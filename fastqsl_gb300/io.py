"""Field input and Q-map output formats of the reference's workflows.

* ``read_sav``  — IDL save files of extrapolated fields, read with
  ``scipy.io.readsav`` and transposed from IDL's (z, y, x) order to the
  tracer's (x, y, z) with x fastest (demo/Q_RKF45CuPy.ipynb cells 1-2: a
  ``twbox`` structure or top-level ``bx/by/bz``; demo/Q_RKF45CuPyStretch.ipynb
  cells 2-3: plus node coordinates ``xa/ya/za`` of a stretched grid).
* ``read_npz``  — NumPy archives of staggered-grid simulation output
  (demo/npzinputRKF45CuPyTwist.ipynb cell 3): face-centred Bx, By, Bz with one
  extra node along their own axis, trimmed to the cell nodes, optionally
  scaled, with the coordinate vectors ``x, y, z``.
* ``write_fits`` / ``read_fits`` — a FITS file with the Q map as the primary
  image and further images as named extensions (demo/Q_RKF45CuPyScott.ipynb
  cell 14 writes q_0 and Bz this way with astropy, which this environment
  does not have; the writer here produces the same header cards).

Arrays come back as float32, Fortran order, shape (nx, ny, nz), ready for
``api.FieldStore`` or the drop-in kernels.
"""
from __future__ import annotations

import numpy as np

__all__ = ["read_sav", "read_npz", "write_fits", "read_fits", "is_uniform_grid"]


def _xfast(a):
    return np.asfortranarray(np.transpose(np.asarray(a), (2, 1, 0)).astype(np.float32))


def read_sav(path, structure="twbox", index=0):
    """Reads Bx, By, Bz (and xa, ya, za when present) from an IDL save file.

    The field is taken from ``<structure>[index]`` when that structure exists
    (the reference's ``a.twbox[0].bx``), else from top-level ``bx, by, bz``.
    Returns (Bx, By, Bz, coords) with coords = (xa, ya, za) float32 or None.
    """
    import scipy.io as sio
    data = sio.readsav(path)
    return _from_sav(data, structure, index)


def _from_sav(data, structure="twbox", index=0):
    keys = {k.lower(): k for k in data.keys()}
    src = None
    if structure and structure.lower() in keys:
        rec = data[keys[structure.lower()]][index]
        fields = {n.lower(): rec[n] for n in rec.dtype.names}
        src = fields
    else:
        src = {k: data[v] for k, v in keys.items()}
    missing = [k for k in ("bx", "by", "bz") if k not in src]
    if missing:
        raise KeyError(f"save file has no {missing} (keys: {sorted(src)})")
    B = [_xfast(src[k]) for k in ("bx", "by", "bz")]
    coords = None
    if all(k in src for k in ("xa", "ya", "za")):
        coords = tuple(np.asarray(src[k]).astype(np.float32).ravel() for k in ("xa", "ya", "za"))
        if [c.size for c in coords] != list(B[0].shape):
            raise ValueError("coordinate lengths do not match the field shape")
    return B[0], B[1], B[2], coords


def read_npz(path, b_scale=1.0, staggered=True):
    """Reads a staggered-grid archive with keys Bx, By, Bz, x, y, z.

    staggered: Bx has one extra node along x, By along y, Bz along z (face
    centred); the first one is dropped, as the reference's npz notebook does.
    Returns (Bx, By, Bz, (x, y, z)), the field multiplied by b_scale (the
    notebook scales by 50); other archive entries are ignored.
    """
    with np.load(path) as z:
        x = z["x"].astype(np.float32)
        y = z["y"].astype(np.float32)
        zz = z["z"].astype(np.float32)
        if staggered:
            Bx = z["Bx"][1:, :, :]
            By = z["By"][:, 1:, :]
            Bz = z["Bz"][:, :, 1:]
        else:
            Bx, By, Bz = z["Bx"], z["By"], z["Bz"]
        B = [np.asfortranarray(b.astype(np.float32) * np.float32(b_scale)) for b in (Bx, By, Bz)]
    if not (B[0].shape == B[1].shape == B[2].shape):
        raise ValueError(f"component shapes differ after trimming: {[b.shape for b in B]}")
    return B[0], B[1], B[2], (x, y, zz)


def is_uniform_grid(coords, rel=0.01):
    """True when every axis is evenly spaced to within `rel` of its smallest
    spacing (the test the reference's stretched notebook uses to pick the
    uniform-spacing index formula, Q_RKF45CuPyStretch.ipynb cell 4)."""
    for a in coords:
        d = np.diff(np.asarray(a, np.float64))
        if (d.max() - d.min()) / d.min() > rel:
            return False
    return True


# --------------------------------------------------------------------------
# FITS (primary image + image extensions), written without astropy
# --------------------------------------------------------------------------
_BLOCK = 2880
_BITPIX = {np.dtype(np.float32): -32, np.dtype(np.float64): -64, np.dtype(np.int16): 16, np.dtype(np.int32): 32,
           np.dtype(np.uint8): 8}


def _card(key, value=None, comment=None):
    """One 80-character header card in the fixed format (value right-aligned
    in columns 11-30 for numbers and logicals, strings quoted from column 11
    and padded to at least 8 characters)."""
    if value is None:
        return key.ljust(80)
    if isinstance(value, bool):
        v = ("T" if value else "F").rjust(20)
    elif isinstance(value, str):
        v = ("'" + value.ljust(8) + "'").ljust(20)
    else:
        v = str(value).rjust(20)
    s = key.ljust(8) + "= " + v
    if comment:
        s += " / " + comment
    return s.ljust(80)[:80]


def _header(cards):
    text = "".join(cards) + _card("END")
    pad = (-len(text)) % _BLOCK
    return (text + " " * pad).encode("ascii")


def _image_cards(a, primary, name=None):
    a = np.asarray(a)
    bitpix = _BITPIX.get(a.dtype)
    if bitpix is None:
        raise TypeError(f"unsupported FITS image dtype {a.dtype}")
    cards = [_card("SIMPLE", True, "conforms to FITS standard") if primary
             else _card("XTENSION", "IMAGE", "Image extension"),
             _card("BITPIX", bitpix, "array data type"),
             _card("NAXIS", a.ndim, "number of array dimensions")]
    # FITS axis 1 is the fastest-varying: the last axis of a C-order array
    for k, n in enumerate(a.shape[::-1]):
        cards.append(_card(f"NAXIS{k + 1}", int(n)))
    if primary:
        cards.append(_card("EXTEND", True))
    else:
        cards.append(_card("PCOUNT", 0, "number of parameters"))
        cards.append(_card("GCOUNT", 1, "number of groups"))
        if name:
            cards.append(_card("EXTNAME", name.upper(), "extension name"))
    return cards


def _data(a):
    a = np.ascontiguousarray(a)
    raw = a.astype(a.dtype.newbyteorder(">")).tobytes()
    return raw + b"\0" * ((-len(raw)) % _BLOCK)


def write_fits(path, primary, extensions=None):
    """Writes `primary` (e.g. the Q map, C order: shape (ny, nx)) as the
    primary image and each (name, array) of `extensions` as an image
    extension, the layout of the reference's Q.fits."""
    with open(path, "wb") as fh:
        fh.write(_header(_image_cards(primary, True)))
        fh.write(_data(primary))
        for name, a in (extensions.items() if isinstance(extensions, dict) else (extensions or [])):
            fh.write(_header(_image_cards(a, False, name)))
            fh.write(_data(a))


def read_fits(path):
    """Reads every image HDU; returns a list of (name, array) with the
    primary HDU named 'PRIMARY'."""
    raw = open(path, "rb").read()
    out = []
    pos = 0
    while pos < len(raw):
        hdr = {}
        while True:
            block = raw[pos:pos + _BLOCK].decode("ascii")
            pos += _BLOCK
            done = False
            for k in range(0, _BLOCK, 80):
                c = block[k:k + 80]
                key = c[:8].strip()
                if key == "END":
                    done = True
                    break
                if c[8:10] == "= ":
                    val = c[10:].split("/")[0].strip() if not c[10:].strip().startswith("'") else \
                        c[10:].strip()[1:].split("'")[0].strip()
                    hdr[key] = val
            if done:
                break
        bitpix = int(hdr["BITPIX"])
        naxis = int(hdr["NAXIS"])
        shape = tuple(int(hdr[f"NAXIS{k}"]) for k in range(naxis, 0, -1))
        dt = {-32: ">f4", -64: ">f8", 16: ">i2", 32: ">i4", 8: "u1"}[bitpix]
        n = int(np.prod(shape)) if naxis else 0
        nbytes = n * np.dtype(dt).itemsize
        arr = np.frombuffer(raw[pos:pos + nbytes], dtype=dt).reshape(shape) if naxis else np.zeros(0)
        pos += nbytes + ((-nbytes) % _BLOCK)
        name = "PRIMARY" if "SIMPLE" in hdr else hdr.get("EXTNAME", f"HDU{len(out)}")
        out.append((name, arr.astype(arr.dtype.newbyteorder("="))))
    return out
