"""The stretched tracer's search tables (field_store.cu: k_stretch_tables;
qsl_field.cuh: stretch_table; bins of one or two intervals as two records
and the node between them, wider bins as ranges) restated in float32 on the
CPU against the reference's bisection (GetIndexBiSearch,
TraceBlineAdaptiveStretch.cu:42-64):
for every coordinate the tables give the cell the bisection gives, including
its answers that are not the containing cell (the cell below near the top of
its last interval, the cell above for the first interval of a 4-node axis).
The GPU tests hold the kernels to the same answers bit for bit; this pins
the scheme itself on many more axes and coordinates."""
import numpy as np
import pytest

f32 = np.float32
BINS_PER_CELL = 4


def reference_bisect(c, a):
    """GetIndexBiSearch: halve [i0, i1] while it spans more than 3 nodes, then
    mid or mid - 1 on one comparison; clamped into [0, n-2]."""
    n = len(a)
    i0, i1, mid = 0, n - 1, n // 2
    while i1 - i0 > 3:
        if c > a[mid]:
            i0 = mid
        else:
            i1 = mid
        mid = (i0 + i1) // 2
    r = mid if c > a[mid] else mid - 1
    return max(min(r, n - 2), 0)


def cell_below(c, a):
    """Largest j in [0, n-2] with a[j] < c (0 if none), in double."""
    lo, hi = 0, len(a) - 2
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if float(a[mid]) < c:
            lo = mid
        else:
            hi = mid - 1
    return lo


def stretch_bin_widening(nb):
    """How far (in bins) each search-table bin is widened on both sides: 1 %
    plus the float rounding of the kernel's bin index (c - a0) * binv, about
    2.4e-7 * nb bins, with margin."""
    return 0.01 + 4e-7 * nb


def build_tables(a):
    n = len(a)
    nb = BINS_PER_CELL * (n - 1)
    rec = [reference_bisect(a[j + 1], a) for j in range(n - 1)]
    a0, w = float(a[0]), (float(a[-1]) - float(a[0])) / nb
    wid = stretch_bin_widening(nb)
    bins = []
    for b in range(nb):
        lo, hi = cell_below(a0 + (b - wid) * w, a), cell_below(a0 + (b + 1 + wid) * w, a)
        hi = max(lo, hi)
        # the device's encoding: one or two intervals as their two records
        # and the node between them (+inf for one), wider ranges as a range
        if hi <= lo + 1:
            bins.append(("pair", f32(a[lo + 1]) if hi > lo else f32(np.inf), rec[lo], rec[hi]))
        else:
            bins.append(("range", lo, hi))
    binv = f32(f32(nb) / f32(a[-1] - a[0]))
    return rec, bins, binv


def table_lookup(c, a, rec, bins, binv, seen=None):
    nb = len(bins)
    b = int(np.trunc(f32(f32(c - a[0]) * binv)))
    entry = bins[min(max(b, 0), nb - 1)]
    if seen is not None:
        seen.add(entry[0])
    if entry[0] == "pair":
        _, node, r_lo, r_hi = entry
        return r_hi if c > node else r_lo
    _, lo, hi = entry
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if c > a[mid]:
            lo = mid
        else:
            hi = mid - 1
    return rec[lo]


def axes(rng):
    for n in (2, 3, 4, 5, 7, 8, 16, 33, 128, 256):
        yield np.cumsum(rng.uniform(0.1, 3.0, n)).astype(f32)              # irregular
        yield (np.cumsum(1.05 ** np.arange(n)) - 50.0).astype(f32)       # geometric
        yield np.linspace(-7.0, 9.0, n).astype(f32)                      # uniform


@pytest.mark.parametrize("seed", [0, 1])
def test_tables_give_the_reference_search_cell(seed):
    rng = np.random.default_rng(seed)
    checked = 0
    seen = set()
    for a in axes(rng):
        a = np.unique(a)
        if len(a) < 2:
            continue
        rec, bins, binv = build_tables(a)
        clo, chi = f32(float(a[0]) + 1e-6), f32(float(a[-1]) - 1e-6)
        cs = np.concatenate([rng.uniform(float(a[0]), float(a[-1]), 400).astype(f32), a,
                             np.nextafter(a, f32(np.inf)), np.nextafter(a, f32(-np.inf))])
        for c in cs:
            c = f32(c)
            c = c if c > a[0] else clo          # the kernel's clamp (stretch_locate)
            c = c if c < a[-1] else chi
            assert table_lookup(c, a, rec, bins, binv, seen) == reference_bisect(c, a), (len(a), float(c))
            checked += 1
    assert checked > 10000
    assert seen == {"pair", "range"}  # both encodings are exercised (the geometric axes have wide bins)


def test_four_node_axis_takes_the_cell_above():
    # the case the tables must reproduce: 4 nodes, a point in the first cell
    a = np.array([0.0, 1.0, 2.0, 3.0], f32)
    assert reference_bisect(f32(0.5), a) == 1
    rec, bins, binv = build_tables(a)
    assert table_lookup(f32(0.5), a, rec, bins, binv) == 1


@pytest.mark.parametrize("bad", [[0.0, 1.0, 1.0], [0.0, 2.0, 1.0], [0.0],
                                 np.array([0.0, 1.0, 1.0 + 1e-9])])  # distinct doubles, one float
def test_trace_stretch_rejects_bad_host_coordinates(bad):
    """The native entry needs strictly increasing node coordinates (the
    search and its tables assume them); host arrays are checked before any
    device work."""
    import torch
    from fastqsl_gb300 import api
    b = torch.zeros(3, 3, 3)
    x = torch.zeros(4)
    with pytest.raises(ValueError):
        api.trace_stretch(b, b, b, [np.asarray(bad), np.arange(3.0), np.arange(3.0)], x, x, x)


def _bisect_vec(c, a):
    """reference_bisect over an array of coordinates."""
    n = len(a)
    i0, i1 = np.zeros(c.shape, np.int64), np.full(c.shape, n - 1)
    mid = np.full(c.shape, n // 2)
    while True:
        act = (i1 - i0) > 3
        if not act.any():
            break
        gt = c > a[mid]
        i0, i1 = np.where(act & gt, mid, i0), np.where(act & ~gt, mid, i1)
        mid = np.where(act, (i0 + i1) // 2, mid)
    r = np.minimum(np.where(c > a[mid], mid, mid - 1), n - 2)
    return np.maximum(r, 0)


def _tables_vec(a, wid):
    n = len(a)
    nb = BINS_PER_CELL * (n - 1)
    rec = _bisect_vec(a[1:], a)
    a0, w = float(a[0]), (float(a[-1]) - float(a[0])) / nb
    b = np.arange(nb)
    below = lambda x: np.clip(np.searchsorted(a.astype(np.float64), x, side="left") - 1, 0, n - 2)  # noqa: E731
    lo, hi = below(a0 + (b - wid) * w), below(a0 + (b + 1 + wid) * w)
    return rec, lo, np.maximum(lo, hi), f32(f32(nb) / f32(a[-1] - a[0]))


def _lookup_vec(c, a, rec, lo, hi, binv):
    b = np.clip(np.trunc((f32(c - a[0]) * binv).astype(f32)).astype(np.int64), 0, len(lo) - 1)
    lo, hi = lo[b].copy(), hi[b].copy()
    while True:
        act = lo < hi
        if not act.any():
            break
        mid = (lo + hi + 1) >> 1
        gt = c > a[np.minimum(mid, len(a) - 1)]
        lo, hi = np.where(act & gt, mid, lo), np.where(act & ~gt, mid - 1, hi)
    return rec[lo]


def test_tables_on_a_long_axis():
    """An irregular axis of ~120,000 nodes (480,000 bins) away from the
    origin, probed at and beside every bin edge and node: there the float
    rounding of the kernel's bin index ((c - a0) * binv) reaches several
    hundredths of a bin, so a fixed 1 % widening of the bins misses the
    reference search's cell for some coordinates (checked below); the
    widening that grows with the bin count gives it for every one."""
    rng = np.random.default_rng(10)
    a = np.unique(np.cumsum(rng.uniform(0.3, 1.7, 120000)).astype(f32) + f32(rng.uniform(-1e4, 1e4)))
    nb = BINS_PER_CELL * (len(a) - 1)
    e = (float(a[0]) + (float(a[-1]) - float(a[0])) * np.arange(1, nb) / nb).astype(f32)
    c = np.concatenate([e, np.nextafter(e, f32(np.inf)), np.nextafter(e, f32(-np.inf)), a[1:-1],
                        np.nextafter(a[1:-1], f32(np.inf))])
    c = np.clip(c, np.nextafter(a[0], f32(np.inf)), np.nextafter(a[-1], f32(-np.inf)))  # the kernel's clamp
    ref = _bisect_vec(c, a)
    got = _lookup_vec(c, a, *_tables_vec(a, stretch_bin_widening(nb)))
    assert (got == ref).all(), int((got != ref).sum())
    fixed = _lookup_vec(c, a, *_tables_vec(a, 0.01))
    assert (fixed != ref).any()  # the case does exercise the rounding
