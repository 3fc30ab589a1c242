"""Measured choice of the tracer's launch configuration.

For a given field store, integrator settings and seed-plane geometry, the
tuner times the main trace on a sample of the workload (a few seed planes
spread evenly over the stack) for each candidate

* seed tile — which seeds a warp's 32 lanes trace together (8x8 tiles give a
  warp a 8x4 patch; 16x16 a 16x2 strip; 4x8 a 4x8 patch),
* resident-block budget — registers per thread sized for 0 (compiler's
  choice), 6, 7, 8, 9 or 10 blocks of 128 threads per SM,
* schedule — static lockstep (one line per thread) against the device work
  queue with 32, 128 or 512 lines per warp refill (lanes refill the moment
  their line ends), on the best tile and budget,

and keeps the fastest.  Results are cached per (device, store layout, field
shape, integrator, plane shape).  tune_batch does the same for the batched
kernels of a QBatch (resident-block budget 6-10, timed on windows of lines
spread over the batch).

The brick edge is not a tuning dimension: an x-pair brick row of 8 records
is one 128-byte line, the unit the L1 charges per warp request, and the
record index is formed with shifts by 3.
"""
from __future__ import annotations

import torch

from . import api

TILES = ((8, 8), (4, 8), (16, 16))
OCCUPANCIES = (0, 6, 7, 8, 9, 10)
QUEUE_CHUNKS = (32, 128, 512)
BATCH_OCCUPANCIES = (6, 7, 8, 9, 10)

_cache: dict = {}


def _key(field, params, n0, n1):
    dev = torch.cuda.get_device_name()
    return (dev, field.layout, tuple(field.shape), int(params.integrator), int(params.tol_law), n0, n1)


def tune_trace(field, xs, ys, zs, params, n0, n1, nplanes, s_len=0.25, tol_coef=1.0, cross_dir=(0.0, 0.0, 1.0),
               sample_planes=4, reps=2, tiles=TILES, occupancies=OCCUPANCIES, chunks=QUEUE_CHUNKS, use_cache=True):
    """Returns {'tile': (ty, tx), 'occupancy': k, 'schedule': 'static' or
    'queue', 'chunk': lines per refill, 'ms': t, 'table': {...}} for the
    fastest candidate on `sample_planes` planes evenly spaced over the stack
    (lines from the bottom and the middle of a cube differ in length and
    spread)."""
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
    queue = torch.zeros(1, dtype=torch.int64, device=xs.device)

    def timed(**kw):
        api.trace(field, sx, sy, sz, **kw)  # warm-up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            api.trace(field, sx, sy, sz, **kw)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    base = dict(params=params, s_len=s_len, tol_coef=tol_coef, cross_dir=cross_dir, out=out)
    table = {}
    orders = {}
    for tile in tiles:
        orders[tile] = api.tile_order(npl, n0, n1, tile[0], tile[1], xs.device)
        for occ in occupancies:
            table[(tile, occ, "static", 0)] = timed(**base, schedule="static", order=orders[tile], occupancy=occ)
    (tile, occ, _, _), _ = min(table.items(), key=lambda kv: kv[1])
    for chunk in chunks:
        table[(tile, occ, "queue", chunk)] = timed(**base, schedule="queue", order=orders[tile], occupancy=occ,
                                                  chunk=chunk, queue=queue)
    (tile, occ, sched, chunk), ms = min(table.items(), key=lambda kv: kv[1])
    res = {"tile": tile, "occupancy": occ, "schedule": sched, "chunk": chunk, "ms": ms,
           "table": {f"{t[0]}x{t[1]}/occ{o}" + (f"/queue{c}" if sc == "queue" else ""): v
                     for (t, o, sc, c), v in table.items()}}
    _cache[key] = res
    return res


def tune_plan(plan, field, xs, ys, zs, params, s_len=0.25, tol_coef=1.0, cross_dir=(0.0, 0.0, 1.0), **kw):
    """Tunes and applies the result to a QMapPlan (its seed order and
    resident-block budget)."""
    res = tune_trace(field, xs, ys, zs, params, plan.n0, plan.n1, plan.nplanes, s_len, tol_coef, cross_dir, **kw)
    ty, tx = res["tile"]
    plan.order = api.tile_order(plan.nplanes, plan.n0, plan.n1, ty, tx, xs.device)
    plan.occupancy = res["occupancy"]
    plan.schedule = res["schedule"]
    if res["schedule"] == "queue":
        plan.chunk = res["chunk"]
    return res


def tune_batch(qb, occupancies=BATCH_OCCUPANCIES, windows=8, window_lines=1 << 15, reps=2):
    """Times the batched main trace of QBatch `qb` at each resident-block
    budget on `windows` windows of lines spread evenly over its line space
    (each window holds whole warps of a few jobs), sets the fastest as
    qb.occupancy (before capture()) and returns {'occupancy': k, 'ms': t,
    'table': {...}}."""
    lines = int(qb.main_lines)
    if lines <= 0:
        return {"occupancy": qb.occupancy, "ms": 0.0, "table": {}}
    w = max(32, min(window_lines, lines // windows) // 32 * 32)
    starts = sorted({(k * lines // windows) // 32 * 32 for k in range(windows)})

    def run(occ):
        for lo in starts:
            qb.main_batch.launch(max_blocks=qb.max_blocks, lo=lo, hi=min(lines, lo + w), occupancy=occ)

    table = {}
    for occ in occupancies:
        run(occ)  # warm-up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            run(occ)
        e1.record()
        torch.cuda.synchronize()
        table[occ] = e0.elapsed_time(e1) / reps
    occ, ms = min(table.items(), key=lambda kv: kv[1])
    qb.occupancy = occ
    return {"occupancy": occ, "ms": ms, "table": {f"occ{o}": v for o, v in table.items()},
            "sample": f"{len(starts)} windows of {w} lines"}
