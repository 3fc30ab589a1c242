"""Measured choice of the tracer's launch configuration.

For a given field store, integrator settings and seed-plane geometry, the
tuner times the main trace on a sample of the workload (a few seed planes
spread evenly over the stack) for each candidate

* seed tile — which seeds a warp's 32 lanes trace together (8x8 tiles give a
  warp a 8x4 patch; 16x16 a 16x2 strip; 4x8 a 4x8 patch),
* resident-block budget — registers per thread sized for 0 (compiler's
  choice), 6, 7, 8, 9 or 10 blocks of 128 threads per SM,

and keeps the fastest.  Results are cached per (device, store layout, field
shape, integrator, plane shape).
"""
from __future__ import annotations

import torch

from . import api

TILES = ((8, 8), (4, 8), (16, 16))
OCCUPANCIES = (0, 6, 7, 8, 9, 10)

_cache: dict = {}


def _key(field, params, n0, n1):
    dev = torch.cuda.get_device_name()
    return (dev, field.layout, tuple(field.shape), int(params.integrator), int(params.tol_law), n0, n1)


def tune_trace(field, xs, ys, zs, params, n0, n1, nplanes, s_len=0.25, tol_coef=1.0, cross_dir=(0.0, 0.0, 1.0),
               sample_planes=4, reps=2, tiles=TILES, occupancies=OCCUPANCIES, use_cache=True):
    """Returns {'tile': (ty, tx), 'occupancy': k, 'ms': t, 'table': {...}}
    for the fastest candidate on `sample_planes` planes evenly spaced over
    the stack (lines from the bottom and the middle of a cube differ in
    length and spread)."""
    key = _key(field, params, n0, n1)
    if use_cache and key in _cache:
        return _cache[key]
    npl = max(1, min(nplanes, sample_planes))
    n = n0 * n1 * npl
    per = n0 * n1
    picks = sorted({round(k * (nplanes - 1) / max(1, npl - 1)) for k in range(npl)}) if npl > 1 else [0]
    idx = torch.cat([torch.arange(k * per, (k + 1) * per, device=xs.device) for k in picks])
    npl, n = len(picks), len(picks) * per
    sx, sy, sz = xs[idx].contiguous(), ys[idx].contiguous(), zs[idx].contiguous()
    out = api.alloc_trace_outputs(n, xs.device)
    table = {}
    for tile in tiles:
        order = api.tile_order(npl, n0, n1, tile[0], tile[1], xs.device)
        for occ in occupancies:
            kw = dict(params=params, s_len=s_len, tol_coef=tol_coef, cross_dir=cross_dir, schedule="static",
                      out=out, order=order, occupancy=occ)
            api.trace(field, sx, sy, sz, **kw)  # warm-up
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                api.trace(field, sx, sy, sz, **kw)
            e1.record()
            torch.cuda.synchronize()
            table[(tile, occ)] = e0.elapsed_time(e1) / reps
    (tile, occ), ms = min(table.items(), key=lambda kv: kv[1])
    res = {"tile": tile, "occupancy": occ, "ms": ms, "table": {f"{t[0]}x{t[1]}/occ{o}": v for (t, o), v in
                                                               table.items()}}
    _cache[key] = res
    return res


def tune_plan(plan, field, xs, ys, zs, params, s_len=0.25, tol_coef=1.0, cross_dir=(0.0, 0.0, 1.0), **kw):
    """Tunes and applies the result to a QMapPlan (its seed order and
    resident-block budget)."""
    res = tune_trace(field, xs, ys, zs, params, plan.n0, plan.n1, plan.nplanes, s_len, tol_coef, cross_dir, **kw)
    ty, tx = res["tile"]
    plan.order = api.tile_order(plan.nplanes, plan.n0, plan.n1, ty, tx, xs.device)
    plan.occupancy = res["occupancy"]
    return res
