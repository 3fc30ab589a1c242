"""Input and output formats of the reference's workflows (fastqsl_gb300.io):
IDL save structures, staggered-grid npz archives, FITS Q maps."""
import json
import os

import numpy as np
import pytest

from fastqsl_gb300 import io

# the reference checkout: $QSL_REFERENCE_ROOT, else `reference` beside the repository
REF = os.environ.get("QSL_REFERENCE_ROOT", os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference"))


def test_fits_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    q = rng.uniform(1, 1e5, size=(100, 240)).astype(np.float32)
    bz = rng.normal(size=(100, 240)).astype(np.float32)
    p = tmp_path / "q.fits"
    io.write_fits(p, q, {"Bz": bz})
    assert os.path.getsize(p) % 2880 == 0
    hdus = io.read_fits(p)
    assert [h[0] for h in hdus] == ["PRIMARY", "BZ"]
    np.testing.assert_array_equal(hdus[0][1], q)
    np.testing.assert_array_equal(hdus[1][1], bz)
    io.write_fits(tmp_path / "d.fits", q.astype(np.float64))
    np.testing.assert_array_equal(io.read_fits(tmp_path / "d.fits")[0][1], q.astype(np.float64))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "Q.fits")), reason="reference checkout not present")
def test_fits_writer_reproduces_reference_file(tmp_path):
    """The reference's Q.fits (written by astropy in Q_RKF45CuPyScott.ipynb
    cell 14): read it, write its images back, get the same bytes."""
    src = os.path.join(REF, "Q.fits")
    hdus = io.read_fits(src)
    assert [h[0] for h in hdus] == ["PRIMARY", "BZ"]
    out = tmp_path / "Q.fits"
    io.write_fits(out, hdus[0][1], {"Bz": hdus[1][1]})
    assert open(out, "rb").read() == open(src, "rb").read()


def _staggered(seed=0, shape=(12, 10, 8)):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    arr = dict(Bx=rng.normal(size=(nx + 1, ny, nz)), By=rng.normal(size=(nx, ny + 1, nz)),
               Bz=rng.normal(size=(nx, ny, nz + 1)), x=np.linspace(0, 1, nx), y=np.linspace(0, 2, ny),
               z=np.linspace(0, 3, nz), num_ghost_cells=np.array(2))
    return arr


def test_npz_trims_staggered_components(tmp_path):
    a = _staggered()
    p = tmp_path / "f.npz"
    np.savez(p, **a)
    Bx, By, Bz, (x, y, z) = io.read_npz(p, b_scale=50.0)
    assert Bx.shape == By.shape == Bz.shape == (12, 10, 8) and Bx.flags.f_contiguous
    np.testing.assert_array_equal(Bx, (a["Bx"][1:].astype(np.float32) * np.float32(50)))
    np.testing.assert_array_equal(Bz, (a["Bz"][:, :, 1:].astype(np.float32) * np.float32(50)))
    np.testing.assert_array_equal(y, a["y"].astype(np.float32))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "demo", "npzinputRKF45CuPyTwist.ipynb")),
                    reason="reference checkout not present")
def test_npz_matches_reference_notebook_cell(tmp_path):
    """Cell 3 of the reference's npz notebook, executed from the notebook
    file on the same archive, gives the same arrays."""
    a = _staggered(1)
    p = tmp_path / "f.npz"
    np.savez(p, **a)
    with open(os.path.join(REF, "demo", "npzinputRKF45CuPyTwist.ipynb")) as f:
        src = "".join(json.load(f)["cells"][3]["source"])
    ns = {"np": np, "npy_arr": np.load(p)}
    exec(compile(src, "npzinputRKF45CuPyTwist.ipynb:cell3", "exec"), ns)
    Bx, By, Bz, (x, y, z) = io.read_npz(p, b_scale=50.0)
    for mine, theirs in ((Bx, ns["Bx"]), (By, ns["By"]), (Bz, ns["Bz"]), (x, ns["x"]), (z, ns["z"])):
        np.testing.assert_array_equal(mine, theirs)


def _idl(a):
    """An (x, y, z) field as readsav returns it: IDL's (z, y, x) order."""
    return np.ascontiguousarray(np.transpose(a, (2, 1, 0)))


def test_sav_structure_and_top_level():
    rng = np.random.default_rng(2)
    B = [rng.normal(size=(6, 5, 4)).astype(np.float32) for _ in range(3)]
    rec = np.empty(1, dtype=[("BX", object), ("BY", object), ("BZ", object)])
    rec[0] = tuple(_idl(b) for b in B)
    got = io._from_sav({"twbox": rec})
    for g, b in zip(got[:3], B):
        np.testing.assert_array_equal(g, b)
        assert g.flags.f_contiguous and g.dtype == np.float32
    assert got[3] is None
    coords = [np.linspace(0, 1, n).astype(np.float32) for n in (6, 5, 4)]
    top = {"bx": _idl(B[0]), "by": _idl(B[1]), "bz": _idl(B[2]), "xa": coords[0], "ya": coords[1], "za": coords[2]}
    got = io._from_sav(top, structure="twbox")
    np.testing.assert_array_equal(got[2], B[2])
    for g, c in zip(got[3], coords):
        np.testing.assert_array_equal(g, c)
    assert io.is_uniform_grid(got[3])
    assert not io.is_uniform_grid((coords[0], coords[1], np.array([0, 1, 3, 7], np.float32)))
