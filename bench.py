"""Benchmark: Q-pixels/s of a full 3-D Q-cube on one GB300.

Workload (one "step"): the 512x512x256 float32 field of 32 sub-surface point
charges (seeded positions at depth 4-20 cells, strengths +-U(0.2, 2)); Q at
every interior cell of the central 256x256x128 sub-box, plane by plane with
z-plane normals (258x258 seeds per plane incl. a one-cell halo for the
central differences, 128 planes traced in one launch), RKF45 with absolute
tolerance 1e-4 and steps in [1e-3, 1] cell, pseudo-lines for the pixels
whose field lies within ~0.6 deg of the plane, FP64 Q assembly.

Forms measured on that workload:
  value      — the fp16 brick store (8^3-cell bricks of x-pair records, a
               float scale per brick; FP32 interpolation of the fp16 node
               values), seeds traced in 8x8 tiles taken through every plane
               of the stack (column order), one line per thread in static
               lockstep, resident blocks per SM from the autotuner
  plain_fp32 — the plain FP32 kernel: SoA float32 field in the caller's
               layout, seeds in row order, one line per thread, compiler's
               register choice; and float32 stores under the headline's own
               schedule, so the fp16 store's share of the gain shows alone
Inputs are resident in HBM during the timed region and larger than L2
(field 805 MB float32, 1.36 GB as fp16 x-pair bricks; outputs ~0.9 GB), so
no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FIELD_SHAPE = [512, 512, 256]
SUB = dict(x0=128, y0=128, z0=64, nx=256, ny=256, nz=128)
S_LEN = 0.25
METRIC = "Q-pixels/s (3-D Q-cube, 512x512x256 field, RKF45 tol 1e-4)"
NPLANES = [SUB["nz"]]  # --planes: fewer z-planes of the same cube (profiling cases)
PLANE0 = [0]  # --plane-offset: first of those planes


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4)
                          if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def workload_name():
    return "qcube-{}-charges32-sub256x256x128-rkf45-tol1e-4".format("x".join(map(str, FIELD_SHAPE)))


def spread_planes(n):
    """n z-plane indices spread evenly over the sub-box's stack."""
    n = max(1, min(SUB["nz"], int(n)))
    return sorted({int(round(v)) for v in np.linspace(0, SUB["nz"] - 1, n)})


def sm_count():
    import ctypes
    from fastqsl_gb300 import _lib
    sms = ctypes.c_int(0)
    _lib.check(_lib.load().qsl_device_sm_count(ctypes.byref(sms)), "qsl_device_sm_count")
    return int(sms.value)


def l1_probe(device, reps=5):
    """The L1 ceiling of 16-byte lane loads (qsl_l1_probe): GB/s with each
    warp request spread over 1-32 128-byte lines, 16 resident blocks of 128
    threads per SM, from a 32 KiB buffer that stays in L1; best of `reps`."""
    import torch
    from fastqsl_gb300 import _lib
    lib = _lib.load()
    buf = torch.zeros(32 << 10, dtype=torch.uint8, device=device)
    sink = torch.zeros(1, dtype=torch.int32, device=device)
    blocks = 16 * sm_count()
    iters = 2048
    st = torch.cuda.current_stream(device)
    out = {}
    for spread in (1, 2, 4, 8, 16, 32):
        run = lambda: _lib.check(lib.qsl_l1_probe(buf.data_ptr(), buf.numel(), spread, blocks, iters,  # noqa
                                                  sink.data_ptr(), st.cuda_stream), "qsl_l1_probe")
        run()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run()
            e1.record(st)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1)
            best = t if best is None else min(best, t)
        out[str(spread)] = blocks * 128 * 8 * iters * 16 / (best / 1e3) / 1e9
    return {"coalesced_gbs": out["4"], "by_spread": out}


def cube_seeds(device, planes=None):
    if planes is None and NPLANES[0] != SUB["nz"]:
        planes = list(range(PLANE0[0], PLANE0[0] + NPLANES[0]))
    from fastqsl_gb300 import api
    s = SUB
    zs = [float(s["z0"] + k) for k in (range(s["nz"]) if planes is None else planes)]
    xs, ys, zz = api.plane_seed_grid(s["x0"] - 1.0, s["x0"] + s["nx"], s["nx"] + 2, s["y0"] - 1.0,
                                     s["y0"] + s["ny"], s["ny"] + 2, zs, device=device)
    return xs, ys, zz, len(zs)


STORE_TYPES = {"h8c": "FieldH8C", "h4b": "FieldH4B", "f4": "FieldF4", "soa": "FieldSoA"}
# --arith: FP32 interpolation (default) or the fp16-x-weight sampler of the
# brick store (opt-in)
ARITHS = {"fast": 1, "w16": 2}


def make_field(device):
    from fastqsl_gb300 import synthetic as S
    spec = S.charges32_512(seed=0, shape=FIELD_SHAPE)
    return S.make_field(spec, device=device, as_numpy=False), spec


def run_ours(args, rank, world):
    import torch
    from fastqsl_gb300 import api, params as P
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    (bx, by, bz), spec = make_field(dev)
    prm = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=ARITHS[args.arith])
    xs, ys, zz, npl = cube_seeds(dev)
    n0, n1 = SUB["ny"] + 2, SUB["nx"] + 2
    qpix = SUB["nx"] * SUB["ny"] * npl
    store = api.FieldStore(bx, by, bz, layout=args.layout)
    plan = api.QMapPlan(n0, n1, npl, device=dev)
    from fastqsl_gb300 import autotune
    if args.no_autotune:
        tuned = {"tile": (8, 8), "occupancy": plan.occupancy_for(store), "schedule": plan.schedule, "chunk": 0,
                 "table": {}}
    else:
        # a quarter of the stack, spread over it: on 8 planes the register
        # budgets of 7 and 8 blocks/SM ranked the other way round from the full cube
        tuned = autotune.tune_plan(plan, store, xs, ys, zz, prm, s_len=S_LEN, sample_planes=max(8, npl // 4))
    stream = torch.cuda.current_stream()

    def step(count=False, ev=None):
        return plan.run(store, xs, ys, zz, prm, s_len=S_LEN, stride=1.0, count_samples=count, kernel_events=ev)

    # warm-up
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # samples per step (device counter) for the roofline
    step(count=True)
    torch.cuda.synchronize()
    samples_main = int(plan.samples_main.item())
    samples_all = int(plan.samples.item())

    from fastqsl_gb300 import replicas
    replicas.barrier()
    torch.cuda.synchronize()
    kev = []
    with ClockSampler(dev.index) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            kev.append(ev)
            step(ev=ev)
        t1.record(stream)
        torch.cuda.synchronize()
    replicas.barrier()
    # every rank traced its own copy of the cube (weak scaling, no exchange
    # on the data path); the job took as long as the slowest rank
    ms = replicas.max_over_ranks(t0.elapsed_time(t1) / args.steps, device=dev)
    k_ms = float(np.mean([a.elapsed_time(b) for a, b in kev]))
    Q = plan.Q

    res = {"ms": ms, "qpix": qpix, "k_ms": k_ms, "samples_main": samples_main, "samples_all": samples_all,
           "sm_count": sm_count(), "l1_probe": l1_probe(dev),
           "clocks": clk.summary(), "autotune": {"tile": list(tuned["tile"]), "occupancy": tuned["occupancy"],
                                                 "schedule": tuned["schedule"], "chunk": tuned["chunk"],
                                                 "sample_ms": tuned["table"]}}
    if rank != 0:
        return res, None

    # ---- plain FP32 kernel (SoA field, static one-line-per-thread grid) ----
    if not args.skip_plain:
        soa = api.FieldStore(bx, by, bz, layout="soa")
        out = plan.main
        for _ in range(2):
            api.trace(soa, xs, ys, zz, prm, s_len=S_LEN, schedule="static", out=out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        reps = max(1, min(3, args.steps))
        for _ in range(reps):
            api.trace(soa, xs, ys, zz, prm, s_len=S_LEN, schedule="static", out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        res["plain_trace_ms"] = e0.elapsed_time(e1) / reps
        # the same trace through the plan's kernel configuration for the ratio
        e0.record(stream)
        for _ in range(reps):
            api.trace(store, xs, ys, zz, prm, s_len=S_LEN, schedule=plan.schedule, out=out, order=plan.order,
                      chunk=plan.chunk, occupancy=plan.occupancy_for(store))
        e1.record(stream)
        torch.cuda.synchronize()
        res["ours_trace_ms"] = e0.elapsed_time(e1) / reps

        def timed_trace(st, p, occ):
            api.trace(st, xs, ys, zz, p, s_len=S_LEN, schedule=plan.schedule, out=out, order=plan.order,
                      chunk=plan.chunk, occupancy=occ)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                api.trace(st, xs, ys, zz, p, s_len=S_LEN, schedule=plan.schedule, out=out, order=plan.order,
                          chunk=plan.chunk, occupancy=occ)
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        # float32 stores under the headline's own schedule (tile/column order,
        # static lockstep): the fp16 store's gain by itself
        f4 = api.FieldStore(bx, by, bz, layout="f4")
        res["same_schedule_f4_ms"] = {str(o): timed_trace(f4, prm.copy(arith=P.ARITH_FAST), o) for o in (0, 6, 8)}
        f4.close()
        res["same_schedule_soa_ms"] = {str(o): timed_trace(soa, prm.copy(arith=P.ARITH_FAST), o) for o in (0, 8)}
        if args.layout == "h4b":
            # the other x-lerp form of the brick store under the same schedule
            other = P.ARITH_FAST_W16 if prm.arith == P.ARITH_FAST else P.ARITH_FAST
            res["other_arith_trace_ms"] = timed_trace(store, prm.copy(arith=other), plan.occupancy_for(store))
        # the reference kernel's design on this GPU: one line per thread in
        # seed order, SoA float32 field, the reference's rounding (corner
        # weights in double), work-queue grid; same settings, one run
        prm_x = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=P.ARITH_EXACT)
        api.trace(soa, xs, ys, zz, prm_x, s_len=S_LEN, schedule="queue", out=out)
        torch.cuda.synchronize()
        e0.record(stream)
        api.trace(soa, xs, ys, zz, prm_x, s_len=S_LEN, schedule="queue", out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        res["exact_trace_ms"] = e0.elapsed_time(e1)
        soa.close()

    # ---- end to end through the public API with host buffers ----
    if not args.skip_e2e:
        hb = [torch.empty(b.shape[::-1], dtype=torch.float32).pin_memory() for b in (bx, by, bz)]
        for h, b in zip(hb, (bx, by, bz)):
            h.copy_(b.permute(2, 1, 0))
        qh = torch.empty(Q.shape, dtype=Q.dtype).pin_memory()
        # two stores and two plans: field k+1's H2D copy and pack overlap
        # field k's trace, and field k's Q copy to the host overlaps field
        # k+1's trace (api.QSeries), with the tuned launch configuration
        series = api.QSeries(tuple(bx.shape), n0, n1, npl, layout=args.layout, device=dev)
        for sp in series.plans:
            sp.order, sp.occupancy, sp.schedule, sp.chunk = plan.order, plan.occupancy, plan.schedule, plan.chunk

        def e2e_run(n):
            # every step: H2D of its field from pinned memory, pack, Q, D2H
            # of Q, each step's copies overlapping its neighbours' traces
            for _ in range(n):
                series.push(*hb, xs, ys, zz, prm, qh, stream=stream, s_len=S_LEN, stride=1.0)
            series.wait(stream)

        e2e_run(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(1, min(8, args.steps))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        e2e_run(reps)
        e1.record(stream)
        torch.cuda.synchronize()
        res["e2e_ms"] = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3) / reps
        res["h2d"] = int(sum(h.numel() * 4 for h in hb))
        res["d2h"] = int(qh.numel() * qh.element_size())
        res["e2e_q_equal"] = bool(torch.equal(qh.to(Q.device).isnan(), Q.isnan()) and
                                  torch.equal(torch.nan_to_num(qh.to(Q.device)), torch.nan_to_num(Q)))
        # the host link by itself: one field's H2D copy alone on the copy
        # stream (the pipeline hides it behind the trace while it is shorter)
        cs = series.up.copy_stream
        h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        h0.record(cs)
        series.up.upload(*hb)
        h1.record(cs)
        torch.cuda.synchronize()
        res["h2d_gbs"] = res["h2d"] / (h0.elapsed_time(h1) * 1e6)
        series.close()

    # ---- accuracy against the FP64 oracle on a seeded sample of cells ----
    if not args.skip_accuracy:
        cubes = {args.arith: Q.cpu().numpy()}
        if args.layout == "h4b":
            # the brick store's other x-lerp form, on the same cells
            oname = "w16" if args.arith == "fast" else "fast"
            plan.run(store, xs, ys, zz, prm.copy(arith=ARITHS[oname]), s_len=S_LEN, stride=1.0)
            cubes[oname] = plan.Q.cpu().numpy()
        res["accuracy"] = accuracy_sample(bx, by, bz, cubes, prm, args.acc_cells)
    store.close()
    return res, Q


def accuracy_sample(bx, by, bz, cubes, prm, ncells):
    """|dlog10 Q| of GPU cubes (name -> Q array) against the FP64 oracle on
    `ncells` seeded cells: each sampled cell's Q is recomputed from its 5-seed
    stencil (and its pseudo-lines when flagged) traced in FP64 on the host."""
    import oracle
    from fastqsl_gb300 import params as P
    from oracle import qassembly as QA
    rng = np.random.default_rng(1234)
    s = SUB
    npl = next(iter(cubes.values())).shape[0]
    ci = rng.integers(0, npl, ncells)
    cj = rng.integers(0, s["ny"], ncells)
    ck = rng.integers(0, s["nx"], ncells)
    B = [b.permute(2, 1, 0).contiguous().cpu().numpy().transpose(2, 1, 0) for b in (bx, by, bz)]
    prm64 = P.absolute_rkf45(tol=prm.tol, h_min=prm.h_min, h_max=prm.h_max, arith=P.ARITH_EXACT)
    # 3x3 stencil planes per cell -> reuse the oracle pipeline on tiny planes
    xs, ys, zs = [], [], []
    for i, j, k in zip(ci, cj, ck):
        z = float(s["z0"] + i)
        x0 = float(s["x0"] + k - 1)
        y0 = float(s["y0"] + j - 1)
        for a in range(3):
            for b in range(3):
                xs.append(x0 + b)
                ys.append(y0 + a)
                zs.append(z)
    xs, ys, zs = (np.array(v, np.float32) for v in (xs, ys, zs))
    tr = lambda a, b, c: oracle.trace_all("port64", B[0], B[1], B[2], a, b, c, s_len=S_LEN,  # noqa: E731
                                          params=prm64)
    Qr = QA.qmap_pipeline(tr, xs, ys, zs, ncells, 3, 3, 1.0)[:, 0, 0]
    out = {}
    for name, Q in cubes.items():
        Qg = Q[ci, cj, ck]
        both = ~np.isnan(Qr) & ~np.isnan(Qg)
        d = np.abs(np.log10(Qg[both]) - np.log10(Qr[both]))
        out[name] = {"cells": int(ncells), "nan_agree": float((np.isnan(Qr) == np.isnan(Qg)).mean()),
                     "median_dlog10Q": float(np.median(d)) if d.size else None,
                     "p99_dlog10Q": float(np.quantile(d, 0.99)) if d.size else None}
    return out


_HOST_FIELD = []


def host_field():
    """The benchmark field on the host (generated once per process)."""
    if not _HOST_FIELD:
        import torch
        (bx, by, bz), _ = make_field("cpu")
        B = [b.numpy() if isinstance(b, torch.Tensor) else b for b in (bx, by, bz)]
        _HOST_FIELD.extend(np.asfortranarray(b) for b in B)
    return _HOST_FIELD


def cpu_baseline(planes, threads=None):
    """The tracing routine (oracle port of the reference's, OpenMP) plus the
    Q assembly on `planes` z-planes of the cube, on the host cores."""
    import oracle
    from fastqsl_gb300 import params as P
    from oracle import qassembly as QA
    B = host_field()
    xs, ys, zz, npl = cube_seeds("cpu", planes=planes)
    xs, ys, zz = xs.numpy(), ys.numpy(), zz.numpy()
    prm = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=P.ARITH_EXACT)
    cores = threads or os.cpu_count()
    tr = lambda a, b, c: oracle.trace_all("port32", B[0], B[1], B[2], a, b, c, s_len=S_LEN, params=prm,  # noqa
                                          threads=cores)
    t = time.perf_counter()
    QA.qmap_pipeline(tr, xs, ys, zz, npl, SUB["ny"] + 2, SUB["nx"] + 2, 1.0, f64=True)
    dt = time.perf_counter() - t
    qpix = SUB["nx"] * SUB["ny"] * npl
    return {"value": qpix / dt, "unit": "Q-pixels/s", "cores": cores, "kind": "port",
            "sample": f"{npl} of {SUB['nz']} z-planes of the same cube ({qpix} Q-pixels), {dt:.1f} s"}


def batched_graph(device, n_fields=64, seed=11, reps=3, acc_fields=8, acc_pixels=40):
    """64 independent fields (4-32 charges; 64^3, 128^3, 192x192x128 or 256^3;
    fp16 bricks or float32 nodes, interleaved), each with an arbitrarily oriented cutting
    plane of 10^3-10^6 seeds (log-uniform), RK4 or RKF45; the whole Q pipeline
    of all 64 captured once into a CUDA graph and replayed.  Accuracy: on
    `acc_fields` of the fields (every 8th), `acc_pixels` seeded interior
    pixels each against the FP64 oracle (each pixel's 3x3 seed stencil on its
    cutting plane, and its pseudo-lines when flagged)."""
    import torch
    from fastqsl_gb300 import api, params as P, synthetic as S
    rng = np.random.default_rng(seed)
    sizes = [(64, 64, 64), (128, 128, 128), (192, 192, 128), (256, 256, 256)]
    specs, stores, keep = [], [], {}
    acc_idx = set(range(0, n_fields, max(1, n_fields // acc_fields))[:acc_fields])
    for k in range(n_fields):
        shape = sizes[int(rng.integers(len(sizes)))]
        spec = S.charges_random(seed * 100 + k, shape, int(rng.integers(4, 33)))
        B = S.make_field(spec, device=device, as_numpy=False)
        layout = "h4b" if rng.random() < 0.5 else "f4"
        fs = api.FieldStore(*B, layout=layout)
        stores.append(fs)
        total = float(np.exp(rng.uniform(np.log(1e3), np.log(1e6))))
        n0 = max(3, int(np.sqrt(total)))
        n1 = max(3, int(total / n0))
        xs, ys, zs, nrm, stride = S.cutting_plane(shape, rng.normal(size=3), n0, n1)
        rkf = rng.random() < 0.5
        prm = P.absolute_rkf45(tol=1e-4) if rkf else P.fixed_rk4(arith=P.ARITH_FAST)
        prm.max_steps = 20000 if not rkf else prm.max_steps
        t = lambda a: torch.from_numpy(a).to(device)  # noqa: E731
        specs.append(dict(field=fs, xs=t(xs), ys=t(ys), zs=t(zs), n0=n0, n1=n1, nplanes=1, params=prm,
                          s_len=0.25 if rkf else 0.1, stride=stride, cross_dir=tuple(float(c) for c in nrm)))
        if k in acc_idx:
            keep[k] = dict(B=[b.cpu().numpy() for b in B], xs=xs, ys=ys, zs=zs, layout=layout, shape=shape,
                           integrator="rkf45" if rkf else "rk4")
        del B
    qb = api.QBatch(specs, device=device)
    from fastqsl_gb300 import autotune
    tuned = autotune.tune_batch(qb)
    qb.capture()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        qb.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    qpix = sum((sp["n0"] - 2) * (sp["n1"] - 2) for sp in specs)
    lines = sum(sp["n0"] * sp["n1"] for sp in specs)
    out = {"fields": n_fields, "seeds": int(lines), "q_pixels": int(qpix), "graph_ms": ms,
           "qpixels_per_s": qpix / (ms / 1e3), "autotune": tuned}
    Qs = {k: qb.jobs[k]["Q"][0].cpu().numpy() for k in keep}
    for fs in stores:
        fs.close()
    del qb
    out["accuracy_vs_fp64"] = batched_accuracy(specs, keep, Qs, acc_pixels)
    return out


def batched_accuracy(specs, keep, Qs, npix, seed=5):
    """|dlog10 Q| of sampled batched-graph pixels against the FP64 oracle:
    per sampled field `npix` seeded interior pixels, each recomputed from its
    3x3 stencil of seeds on the field's cutting plane (and its pseudo-lines
    when flagged) traced in FP64 with the job's own integrator settings."""
    import oracle
    from fastqsl_gb300 import params as P
    from oracle import qassembly as QA
    rng = np.random.default_rng(seed)
    per, d_all, nan_all = {}, [], []
    for k, kv in sorted(keep.items()):
        sp = specs[k]
        n0, n1 = sp["n0"], sp["n1"]
        Q = Qs[k]
        ci = rng.integers(0, n0 - 2, npix)
        cj = rng.integers(0, n1 - 2, npix)
        gx, gy, gz = (a.reshape(n0, n1) for a in (kv["xs"], kv["ys"], kv["zs"]))
        sx = np.concatenate([gx[i:i + 3, j:j + 3].ravel() for i, j in zip(ci, cj)])
        sy = np.concatenate([gy[i:i + 3, j:j + 3].ravel() for i, j in zip(ci, cj)])
        sz = np.concatenate([gz[i:i + 3, j:j + 3].ravel() for i, j in zip(ci, cj)])
        prm64 = sp["params"].copy(arith=P.ARITH_EXACT)
        B = kv["B"]
        tr = lambda a, b, c: oracle.trace_all("port64", B[0], B[1], B[2], a, b, c,  # noqa: E731
                                              cross_dir=sp["cross_dir"], s_len=sp["s_len"], params=prm64)
        Qr = QA.qmap_pipeline(tr, sx, sy, sz, npix, 3, 3, sp["stride"], cross_dir=sp["cross_dir"])[:, 0, 0]
        Qg = Q[ci, cj]
        both = ~np.isnan(Qr) & ~np.isnan(Qg)
        d = np.abs(np.log10(Qg[both]) - np.log10(Qr[both]))
        nan_agree = np.isnan(Qr) == np.isnan(Qg)
        per[str(k)] = {"layout": kv["layout"], "shape": "x".join(map(str, kv["shape"])),
                       "integrator": kv["integrator"], "nan_agree": float(nan_agree.mean()),
                       "median_dlog10Q": float(np.median(d)) if d.size else None}
        d_all.append(d)
        nan_all.append(nan_agree)
    d = np.concatenate(d_all) if d_all else np.zeros(0)
    return {"fields": len(keep), "pixels": int(sum(len(a) for a in nan_all)),
            "nan_agree": float(np.concatenate(nan_all).mean()) if nan_all else None,
            "median_dlog10Q": float(np.median(d)) if d.size else None,
            "p99_dlog10Q": float(np.quantile(d, 0.99)) if d.size else None, "per_field": per}


def forms(device, planes=16):
    """The other forms of the path, each timed with CUDA events on its own
    workload: on 16 mid-cube planes of the benchmark field (fp16 bricks) the
    Q map by finite differences + pseudo-lines (the headline pipeline) and by
    finite differences + Scott q_perp where they fail (hybrid), the main
    trace with and without the twist integral (current from the GPU curl),
    the Scott deviation-vector tracer alone on 2 planes (seeds in 8x8 tiles);
    and the stretched-grid
    tracer on a 256x256x128 grid, 1024x1024 seeds: the cell search with z
    spacing growing 1 % per cell, the uniform-spacing formula on uniform
    spacing."""
    import torch
    from fastqsl_gb300 import api, params as P, synthetic as S
    from fastqsl_gb300.fastqslpy import FastQSL

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    (bx, by, bz), _ = make_field(device)
    prm = P.absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=P.ARITH_FAST)
    mid = SUB["nz"] // 2 - planes // 2
    xs, ys, zz, npl = cube_seeds(device, planes=list(range(mid, mid + planes)))
    n0, n1 = SUB["ny"] + 2, SUB["nx"] + 2
    qpix = SUB["nx"] * SUB["ny"] * npl
    store = api.FieldStore(bx, by, bz, layout="h4b")
    res = {"workload": f"{npl} mid-cube planes ({qpix} Q-pixels) of the benchmark field, fp16 bricks"}
    plan = api.QMapPlan(n0, n1, npl, device=device)
    ms = timed(lambda: plan.run(store, xs, ys, zz, prm, s_len=S_LEN, stride=1.0))
    res["q_fd_pseudo"] = {"ms": ms, "qpixels_per_s": qpix / ms * 1e3}
    Qa = plan.Q.clone()
    hyb = api.QMapPlan(n0, n1, npl, device=device, hybrid=True)
    ms = timed(lambda: hyb.run(store, xs, ys, zz, prm, s_len=S_LEN, stride=1.0))
    Qb = hyb.Q
    both = torch.isfinite(Qa) & torch.isfinite(Qb) & (Qa > 0) & (Qb > 0)
    d = (torch.log10(Qa[both]) - torch.log10(Qb[both])).abs()
    res["q_hybrid_scott"] = {"ms": ms, "qpixels_per_s": qpix / ms * 1e3, "scott_pixels": int(hyb.hcount.item()),
                             "nan_pixels": int((~torch.isfinite(Qb)).sum().item()),
                             "nan_pixels_fd_pseudo": int((~torch.isfinite(Qa)).sum().item()),
                             "median_dlog10Q_vs_fd_pseudo": float(d.median().item()) if d.numel() else None}
    del hyb
    order = api.tile_order(npl, n0, n1, 8, 8, device)
    out = api.alloc_trace_outputs(xs.numel(), device, twist=True)
    ax = [torch.arange(n, dtype=torch.float32, device=device) for n in bx.shape]
    cur = [api.as_xfast(c.float()) for c in FastQSL.curl_of_B_grid(bx, by, bz, *ax)]
    cnt = torch.zeros(1, dtype=torch.int64, device=device)
    kw = dict(s_len=S_LEN, schedule="static", out=out, order=order)
    f4 = api.FieldStore(bx, by, bz, layout="f4")

    def best(fn):
        # each form at its best register budget of 6, 7 or 8 blocks/SM (the
        # twist kernels hold more live values than the plain trace)
        return min((timed(lambda: fn(o)), o) for o in (6, 7, 8))

    for name, st in (("h4b", store), ("f4", f4)):
        cs = api.FieldStore(*cur, layout=name)
        ms0, o0 = best(lambda o: api.trace(st, xs, ys, zz, prm, occupancy=o, **kw))
        ms1, o1 = best(lambda o: api.trace(st, xs, ys, zz, prm, curB=cur, occupancy=o, **kw))
        ms2, o2 = best(lambda o: api.trace(st, xs, ys, zz, prm, curB=cs, occupancy=o, **kw))
        cnt.zero_()
        api.trace(st, xs, ys, zz, prm, curB=cs, samples=cnt, occupancy=o2, **kw)
        torch.cuda.synchronize()
        res[f"trace_twist_{name}"] = {"lines": int(xs.numel()), "ms_without": ms0, "ms_with_current_arrays": ms1,
                                      "ms_with_current_store": ms2, "samples_with": int(cnt.item()),
                                      "blocks_per_sm": {"without": o0, "current_arrays": o1, "current_store": o2}}
        cs.close()
    f4.close()
    del cur, out
    m = 2 * n0 * n1
    sx, sy, sz = xs[:m].contiguous(), ys[:m].contiguous(), zz[:m].contiguous()
    so = api.alloc_scott_outputs(m, device)
    sprm = P.reference_scott(arith=P.ARITH_FAST).copy(tol=1e-4, h_min=1e-3, h_max=1.0)
    sorder = api.tile_order(2, n0, n1, 8, 8, device)
    for g in ("analytic", "fd"):
        cnt.zero_()
        ms = timed(lambda: api.trace_scott(store, sx, sy, sz, sprm, s_len=S_LEN, grad=g, out=so, order=sorder))
        api.trace_scott(store, sx, sy, sz, sprm, s_len=S_LEN, grad=g, out=so, samples=cnt, order=sorder)
        torch.cuda.synchronize()
        res[f"scott_{g}"] = {"lines": m, "ms": ms, "samples": int(cnt.item()),
                             "g_samples_per_s": cnt.item() / (ms * 1e6)}
    store.close()
    shape = (256, 256, 128)
    spec = S.bipole4_stretch(3, shape)
    gx = torch.linspace(-5.5, 5.5, 1024, device=device)
    gy = torch.linspace(-4.5, 4.5, 1024, device=device)
    Y, X = torch.meshgrid(gy, gx, indexing="ij")
    px, py = X.reshape(-1).contiguous(), Y.reshape(-1).contiguous()
    sp = P.reference_stretch(arith=P.ARITH_FAST).copy(tol_law=P.TOL_ABSOLUTE, tol=1e-5, h_min=1e-4, h_max=0.05)
    # the search on a grid whose z spacing grows 1 % per cell; the uniform
    # formula (flag_uni) on the same box with uniform spacing, where it holds
    for uni, ratio in ((False, 1.01), (True, 1.0)):
        coords = S.stretched_axes(shape, z_ratio=ratio)
        Bs = [torch.from_numpy(b).to(device) for b in S.make_field_coords(spec, *coords)]
        pz = torch.full_like(px, float(coords[2][1]) * 0.5)
        cnt.zero_()
        api.trace_stretch(*Bs, coords, px, py, pz, sp, s_len=0.01, uni=uni, samples=cnt)
        torch.cuda.synchronize()
        tiles = api.tile_order(1, 1024, 1024, 8, 8, device)
        # static lockstep over the register budgets (4, 5 = the default, 6
        # blocks per SM) in seed rows and 8x8 tiles; the work queue at the
        # default budget in tiles
        cfgs = [("static", o, name, order) for o in (4, 5, 6) for name, order in (("rows", None), ("tiles", tiles))]
        cfgs.append(("queue", 5, "tiles", tiles))
        cfg_ms = {f"{sch}/occ{o}/{name}": timed(lambda: api.trace_stretch(*Bs, coords, px, py, pz, sp, s_len=0.01,
                                                                          uni=uni, occupancy=o, schedule=sch,
                                                                          order=order))
                  for sch, o, name, order in cfgs}
        ms = min(cfg_ms.values())
        res["stretch_" + ("uniform_formula" if uni else "search")] = {
            "grid": "x".join(map(str, shape)), "z_ratio": ratio, "lines": int(px.numel()), "ms": ms,
            "ms_by_launch": cfg_ms, "samples": int(cnt.item()), "g_samples_per_s": cnt.item() / (ms * 1e6)}
    return res


def serving_accuracy(alone, device, server, nreq=4, npix=30, seed=9):
    """|dlog10 Q| of `nreq` isolated serving results (the first requests of
    the stream, each on its own resident field) against the FP64 oracle:
    `npix` seeded interior pixels each, recomputed from the pixel's 3x3 seed
    stencil on the request's plane (and its pseudo-lines when flagged) with
    the request's tolerance; the field is regenerated from its seeded spec
    for the host."""
    import oracle
    from fastqsl_gb300 import params as P, serving, synthetic as S
    from oracle import qassembly as QA
    rng = np.random.default_rng(seed)
    d_all, nan_all, per = [], [], {}
    for rid in sorted(alone)[:nreq]:
        r, Q = alone[rid]
        k = int(r.field[1:])
        B = [b.cpu().numpy() for b in S.make_field(S.charges_tube(k, (384, 384, 256), n_charges=8),
                                                    device=device, as_numpy=False)]
        xs, ys, zs, nrm = serving.seeds_on_device(r, device)
        g = [a.cpu().numpy().reshape(r.nplanes, r.n0, r.n1) for a in (xs, ys, zs)]
        cp = rng.integers(0, r.nplanes, npix)
        ci = rng.integers(0, r.n0 - 2, npix)
        cj = rng.integers(0, r.n1 - 2, npix)
        st = [np.concatenate([a[p, i:i + 3, j:j + 3].ravel() for p, i, j in zip(cp, ci, cj)]) for a in g]
        prm = P.absolute_rkf45(tol=r.tol, h_min=server.h_min, h_max=server.h_max, arith=P.ARITH_EXACT)
        tr = lambda a, b, c: oracle.trace_all("port64", B[0], B[1], B[2], a, b, c, cross_dir=nrm,  # noqa: E731
                                              s_len=server.s_len, params=prm)
        Qr = QA.qmap_pipeline(tr, *st, npix, 3, 3, r.spacing, cross_dir=nrm)[:, 0, 0]
        Qg = Q[cp, ci, cj]
        both = ~np.isnan(Qr) & ~np.isnan(Qg)
        d = np.abs(np.log10(Qg[both]) - np.log10(Qr[both]))
        per[str(rid)] = {"seeds": r.seeds, "tol": r.tol, "median_dlog10Q": float(np.median(d)) if d.size else None}
        d_all.append(d)
        nan_all.append(np.isnan(Qr) == np.isnan(Qg))
    d = np.concatenate(d_all) if d_all else np.zeros(0)
    return {"requests": len(per), "pixels": int(sum(len(a) for a in nan_all)),
            "nan_agree": float(np.concatenate(nan_all).mean()) if nan_all else None,
            "median_dlog10Q": float(np.median(d)) if d.size else None,
            "p99_dlog10Q": float(np.quantile(d, 0.99)) if d.size else None, "per_request": per}


def serving_sweep(device, count=512):
    """8 resident 384x384x256 fields; Poisson streams of `count` Q-map
    requests (tol 1e-3/1e-4/1e-5) at fractions of the batched (whole-batch
    launches, all requests at once) saturated rate, served with windowed bulk
    traces; p50/p99 latency against each request's isolated solve, beside
    what an ideal fluid scheduler reaches on the same stream.  Two mixes: the
    serving configuration's 10^4-4x10^6 seeds (log-uniform), and small
    requests of 10^4-3x10^4 seeds, where even the ideal scheduler's p99 at
    80 % load is within 2x isolated only because no request fills the GPU
    alone."""
    from fastqsl_gb300 import serving
    fields = serving.make_fields(n_fields=8, shape=(384, 384, 256), device=device)
    srv = serving.QServer(fields, hbm_budget=48 << 30, streams=3, max_batch=16)
    whole = serving.QServer(fields, hbm_budget=48 << 30, streams=3, max_batch=16, chunk_lines=0)
    alone = {}
    out = serving.sweep(srv, (384, 384, 256), count=count, fractions=(0.5, 0.8), batched_server=whole,
                        alone_out=alone)
    out["mix"] = "1e4-4e6 seeds, log-uniform"
    out["accuracy_vs_fp64"] = serving_accuracy(alone, device, srv)
    small = serving.sweep(srv, (384, 384, 256), count=count, fractions=(0.5, 0.8), batched_server=whole,
                          seeds_range=(1e4, 3e4))
    small["mix"] = "1e4-3e4 seeds, log-uniform"
    out["small_requests"] = small
    for fs in fields.values():
        fs.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--layout", default="h4b", choices=["h8c", "h4b", "f4", "soa"])
    ap.add_argument("--arith", default="fast", choices=list(ARITHS),
                    help="fast: FP32 interpolation; w16: fp16 x weights (h4b only)")
    ap.add_argument("--cpu-planes", type=int, default=32)
    ap.add_argument("--ref-planes", type=int, default=8, help="z-planes per step of --impl reference")
    ap.add_argument("--acc-cells", type=int, default=2000)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch configuration (profiling)")
    ap.add_argument("--skip-serving", action="store_true")
    ap.add_argument("--skip-forms", action="store_true")
    ap.add_argument("--forms-only", action="store_true", help="only the forms section (profiling)")
    ap.add_argument("--batched-only", action="store_true", help="only the batched-graph section (profiling)")
    ap.add_argument("--planes", type=int, default=SUB["nz"], help="z-planes of the cube (profiling: fewer)")
    ap.add_argument("--plane-offset", type=int, default=0, help="first z-plane with --planes")
    ap.add_argument("--field-nz", type=int, default=FIELD_SHAPE[2],
                    help="z nodes of the field (512: a 512^3 field around the same central Q-cube)")
    args = ap.parse_args()
    if args.field_nz != FIELD_SHAPE[2]:
        # a taller field: the Q sub-box stays central (z offset by half the
        # extra height), the charges keep their depths below z = 0
        nz = max(SUB["nz"] + 2, int(args.field_nz))
        SUB["z0"] += (nz - FIELD_SHAPE[2]) // 2
        FIELD_SHAPE[2] = nz
    NPLANES[0] = max(1, min(SUB["nz"], args.planes))
    PLANE0[0] = max(0, min(SUB["nz"] - NPLANES[0], args.plane_offset))

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    if args.forms_only or args.batched_only:
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
        print(json.dumps({"forms": forms(dev)} if args.forms_only else {"batched_graph": batched_graph(dev)}))
        return

    if args.impl == "reference":
        if rank != 0:
            return
        # each step is a bounded sample of the cube: `--ref-planes` z-planes
        # spread evenly over the 128-plane stack, shifted from step to step,
        # timed whole; the rate and ms_per_step are those of that sample
        npl = max(1, min(SUB["nz"], args.ref_planes))
        gap = SUB["nz"] // npl

        def planes_of(k):
            return sorted({(j * gap + (k * 5) % gap) % SUB["nz"] for j in range(npl)})

        for k in range(args.warmup):
            cpu_baseline([planes_of(k)[0]], None)
        per, wall = [], []
        for k in range(args.steps):
            t = time.perf_counter()
            per.append(cpu_baseline(planes_of(k), None))
            wall.append(time.perf_counter() - t)
        qpix_step = SUB["nx"] * SUB["ny"] * npl
        v = qpix_step * len(per) / float(sum(wall))
        line = {"metric": METRIC, "value": v, "unit": "Q-pixels/s", "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(wall)) * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": workload_name(),
                           "step": f"{npl} of the {SUB['nz']} z-planes ({qpix_step} Q-pixels), spread evenly "
                                   f"over the stack and shifted each step"},
                "cpu_baseline": {**per[-1], "value": v,
                                 "sample": f"{npl} z-planes per step ({qpix_step} Q-pixels), {args.steps} steps"},
                "e2e": {"value": v, "unit": "Q-pixels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res, _ = run_ours(args, rank, world)
    if rank != 0:
        return
    peak, peak_kind = peaks()
    ms = res["ms"]
    from fastqsl_gb300 import replicas
    value = replicas.whole_job_rate(res["qpix"], ms, world)
    fp16 = args.layout in ("h4b", "h8c")
    k_s = res["k_ms"] / 1e3
    # algorithmic bytes per field sample: 8 corners x 3 components (fp16: 48 B,
    # float32: 96 B); the bytes the sampler's loads move through L1 per
    # sample: four 16-byte x-pair records (h4b), 32 + 16 B (h8c), eight
    # 16-byte nodes (f4), 24 4-byte words (soa)
    alg_bytes = 48 if fp16 else 96
    l1_bytes = {"h4b": 64, "h8c": 48, "f4": 128, "soa": 96}[args.layout]
    l1 = res["l1_probe"]
    l1_achieved = res["samples_main"] * l1_bytes / k_s / 1e9
    hbm_achieved = res["samples_main"] * alg_bytes / k_s / 1e9
    acc = res.get("accuracy", {})
    line = {
        "metric": METRIC, "value": value, "unit": "Q-pixels/s",
        "accuracy_vs_fp64": acc.get(args.arith) if acc else None,
        "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (fp16 field storage)" if fp16 else "f32",
        "data": "synthetic",
        "config": {"workload": workload_name(),
                   "field": "x".join(map(str, FIELD_SHAPE)), "qcube": "256x256x128", "layout": args.layout,
                   "interpolation": "FP32 weights and lerps of fp16 node values" if args.arith == "fast"
                   else "fp16 x weights (opt-in sampler)",
                   "h": [1e-3, 1.0], "planes": NPLANES[0], "l2": "inputs larger than L2 (no flush)"},
        "gpu_launches": None,
        "clocks": res["clocks"],
        "roofline": {
            "bound": "l1", "achieved": l1_achieved, "peak": l1["coalesced_gbs"], "unit": "GB/s",
            "frac": l1_achieved / l1["coalesced_gbs"],
            # DRAM bytes per launch: ncu's dram__bytes_read.sum + write.sum of
            # the full-size main trace (one-pass capture: 1.18 GB read + 0.70 GB
            # written for 14.82 G samples), per this launch's samples
            "traffic": (1.884e9 / 14.816e9) * res["samples_main"] if args.layout == "h4b" else None,
            "kernel": f"k_trace_fast<static, {STORE_TYPES[args.layout]}> (main trace)",
            "note": (f"L1 bytes the field gathers load = {l1_bytes} B x {res['samples_main']} field samples per "
                     f"launch / {res['k_ms']:.2f} ms (CUDA events on the launch stream); peak = qsl_l1_probe in "
                     f"this run: 16-byte lane loads from an L1-resident buffer, coalesced (4 lines per warp "
                     f"request); the tracer's requests are scattered gathers, so its L1 wavefronts per byte "
                     f"exceed the probe's"),
            "l1_probe_gbs_by_lines_per_request": l1["by_spread"],
            "hbm": {"achieved": hbm_achieved, "peak": peak, "unit": "GB/s", "frac": hbm_achieved / peak,
                    "peak_kind": peak_kind,
                    "note": f"algorithmic {alg_bytes} B per sample; above 1 because the gathers hit L1/L2, "
                            f"DRAM traffic is the 'traffic' figure"},
        },
    }
    # FP32 flop view: 75 flops per normalised field sample (18 weights, 24 FMA,
    # 9 to normalise) plus 130 per RKF45 step for the combine and error
    # estimate, one step per 6 samples.  Nominal peak from the device's SM
    # count (128 FP32 lanes x 2 flops per SM per clock at 2.07 GHz); no
    # measured FP32 figure exists for this GPU.
    flops = res["samples_main"] * (75.0 + 130.0 / 6.0)
    fp32_peak = res["sm_count"] * 128 * 2 * 2.07e9 / 1e12
    line["roofline"]["flops"] = {"achieved": flops / k_s / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                                 "frac": flops / k_s / 1e12 / fp32_peak, "peak_kind": "nominal",
                                 "sm_count": res["sm_count"]}
    line["roofline"]["limiter"] = ("SM issue, the FMA pipe and the L1 data pipe together (ncu on 32 mid-cube "
                                   "planes: issue active ~74 %, FMA pipe ~64 % of its cycles, L1 LSU wavefronts "
                                   "~76 % of peak)")
    # launches per step: main trace, qcalc, flag_count, tile_scan, cook_write,
    # pseudo trace, qcut, qmerge (+ 2 memsets of the queue counters)
    line["gpu_launches"] = 8 * args.steps
    line["config"]["autotune"] = res["autotune"]
    at = res["autotune"]
    sched = "static lockstep" if at["schedule"] == "static" else f"work queue, {at['chunk']} lines per refill"
    line["config"]["schedule"] = (f"{sched}, {at['tile'][0]}x{at['tile'][1]} seed tiles in column order, "
                                  f"occupancy {at['occupancy']} ({'default' if args.no_autotune else 'autotuned'})")
    if acc:
        line["accuracy_vs_fp64_all_forms"] = acc
    if "plain_trace_ms" in res:
        line["plain_fp32"] = {
            "trace_ms": res["plain_trace_ms"], "ours_trace_ms": res["ours_trace_ms"],
            "speedup": res["plain_trace_ms"] / res["ours_trace_ms"],
            "plain": "SoA float32 field, seeds in row order, compiler's registers, same fast stepper",
            "same_schedule_f4_trace_ms": res["same_schedule_f4_ms"],
            "same_schedule_soa_trace_ms": res["same_schedule_soa_ms"],
            "speedup_vs_same_schedule_f32": min(res["same_schedule_f4_ms"].values()) / res["ours_trace_ms"],
            "reference_design_trace_ms": res.get("exact_trace_ms"),
            "speedup_vs_reference_design": res["exact_trace_ms"] / res["ours_trace_ms"]
            if res.get("exact_trace_ms") else None}
        if "other_arith_trace_ms" in res:
            line["plain_fp32"]["other_arith"] = {"arith": "w16" if args.arith == "fast" else "fast",
                                                 "trace_ms": res["other_arith_trace_ms"]}
    if "e2e_ms" in res:
        line["e2e"] = {"value": res["qpix"] / (res["e2e_ms"] / 1e3), "unit": "Q-pixels/s",
                       "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                       "q_equals_device_run": res["e2e_q_equal"], "h2d_gb_per_s_alone": res["h2d_gbs"]}
    if not args.skip_batched:
        import torch
        line["batched_graph"] = batched_graph(torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0))))
    if not args.skip_forms:
        import torch
        line["forms"] = forms(torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0))))
    if not args.skip_serving:
        import torch
        line["serving"] = serving_sweep(torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0))))
    if not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(spread_planes(args.cpu_planes))
    line["samples_per_step"] = res["samples_all"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
