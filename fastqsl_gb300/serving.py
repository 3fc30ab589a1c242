"""Resident-field Q-map serving with continuous batching.

Fields stay on the device (FieldStore).  Requests name a field, a stack of
seed planes (an arbitrarily oriented plane, or several parallel ones = a
sub-box) and an RKF45 tolerance.  The scheduler loop:

* completes finished batches (a CUDA event per batch; results were copied to
  pinned host memory on the batch's stream) and returns their memory to the
  HBM budget;
* sorts requests into size classes; per class, admits waiting requests in
  arrival order while their device memory fits in what the budget has left,
  up to the class's batch size and in-flight limit;
* launches every newly admitted group as one batch (PlaneQBatch, the native
  qsl_qmap_batch: seed grids, tile orders and job tables built by the C++
  library in one workspace allocation; one main-trace launch and one
  pseudo-line launch for all of them) on one of the class's
  CUDA streams, so a batch starts while earlier ones are still on the GPU and
  their work overlaps on the device.  Smaller classes run on higher-priority
  streams: their blocks are dispatched ahead of a large batch's remaining
  blocks, and larger classes keep at most `big_blocks_per_sm` of the 8
  resident block slots per SM, so a small request finds free slots at once
  instead of waiting for a large batch's blocks to retire;
* runs the main trace of larger classes' batches as windows of
  `chunk_lines` lines (qsl_batch_run_window), at most `max_chunks` windows
  on the device at a time and `chunks_when_interactive` while a batch of the
  smallest class is in flight, so a small request shares the GPU with at
  most that many windows of bulk work, not with whole bulk batches; the
  batch's Q assembly runs after its last window.

Nothing in the loop synchronises the device: allocations come from the
caching allocator on the batch's stream, the job table is copied
asynchronously from pinned memory, completion is polled.  A request's result
does not depend on what it was batched with (each line is traced by one
thread with its job's settings; tests check alone == in the mix bit for bit).
"""
from __future__ import annotations

import collections
import gc
import math
import time
from dataclasses import dataclass, field as dc_field

import numpy as np
import torch

from . import api
from .params import absolute_rkf45


@dataclass
class QRequest:
    """A Q-map request: nplanes parallel (n0, n1) seed planes on `field`,
    plane k offset by k*spacing along `normal` from `center`."""
    rid: int
    field: str
    n0: int
    n1: int
    nplanes: int = 1
    center: tuple = (0.0, 0.0, 0.0)
    normal: tuple = (0.0, 0.0, 1.0)
    spacing: float = 1.0
    tol: float = 1e-4
    arrival: float = 0.0          # seconds after the stream starts (run_stream)
    # filled by the server
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    result: np.ndarray | None = None
    meta: dict = dc_field(default_factory=dict)

    @property
    def seeds(self):
        return self.n0 * self.n1 * self.nplanes

    @property
    def qpixels(self):
        return self.nplanes * (self.n0 - 2) * (self.n1 - 2)

    @property
    def latency(self):
        return self.t_done - self.t_submit


def request_bytes(req: QRequest) -> int:
    """Device bytes a request holds while in flight (batch buffers: main
    trace outputs, order, seeds, the pseudo-line buffers sized for every
    interior pixel, Q and the compaction workspace)."""
    n, m = req.seeds, req.qpixels
    # (+ the 256-byte alignment of each of the job's ~60 arrays and its
    # share of the job tables)
    return int(n * (72 + 8 + 4 + 12 + 4) + m * (4 * (72 + 8 + 12) + 8 + 8 + 8 + 8) + (n // 1024 + 1) * 12 + 20480)


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _unit(a):
    r = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
    return (a[0] / r, a[1] / r, a[2] / r)


def plane_axes(normal):
    """An orthonormal frame (n, u, v) of a plane with normal `normal`: u
    across the coordinate axis least aligned with n, v = n x u (plain
    floats: called once per request on the serving path)."""
    n = _unit(tuple(float(c) for c in normal))
    k = min(range(3), key=lambda i: abs(n[i]))
    e = tuple(1.0 if i == k else 0.0 for i in range(3))
    u = _unit(_cross(n, e))
    return n, u, _cross(n, u)


def seeds_on_device(req: QRequest, device, stream=None):
    """Seeds of the request's planes, built on the device in one launch (no
    host copy): plane k, row i, column j at center + (j - (n1-1)/2) s u +
    (i - (n0-1)/2) s v + k s n (api.plane_seeds), on `stream` (default:
    the current stream)."""
    n, u, v = plane_axes(req.normal)
    xs, ys, zs = api.plane_seeds(req.center, n, u, v, req.spacing, req.n0, req.n1, req.nplanes, device=device,
                                 stream=stream)
    return xs, ys, zs, n


class _Flight:
    """One admitted batch: its requests, buffers, stream, pinned results and
    completion event (None until the post-trace steps are queued); a chunked
    batch also keeps the next window's first line and its windows' events."""

    def __init__(self, reqs, qb, cls, stream, nbytes):
        self.reqs, self.qb, self.cls, self.stream, self.nbytes = reqs, qb, cls, stream, nbytes
        self.hosts, self.event = [], None
        self.next_lo, self.lines, self.nwin = 0, 0, 0
        self.ready = None          # recorded on `stream` once the batch's tables are queued
        self.windows = []          # events of windows not yet seen complete
        self.last = {}             # window stream index -> event of this batch's last window there

    def windows_in_flight(self):
        self.windows = [e for e in self.windows if not e.query()]
        return len(self.windows)


class QServer:
    """Continuous-batching Q-map server over resident fields.

    fields: {name: FieldStore}.  hbm_budget: bytes the in-flight requests may
    hold; a request larger than the whole budget is rejected at submit.
    streams: CUDA streams batches rotate over (overlap on the device); each
    class gets at least as many as it may have batches in flight.
    max_batch: requests per batch."""

    # size classes: (upper bound on seeds, requests per batch, batches in flight)
    # (larger requests fill the GPU alone: batching them only makes each
    # wait for its batch mates; the smallest class runs small batches, many
    # in flight, each on its own stream: 2 per batch with 12 in flight held
    # the small-request mix's p99 at 5.8x isolated at 80 % load against
    # 11.3x for 8 per batch with 4 in flight on 3 streams, at a higher
    # saturated rate)
    CLASSES = ((1.5e5, 2, 12), (1.2e6, 2, 3), (float("inf"), 1, 3))

    def __init__(self, fields, hbm_budget=16 << 30, streams=2, max_batch=None, s_len=0.25, h_min=1e-3, h_max=1.0,
                 tile=(8, 8), device="cuda", classes=None, big_blocks_per_sm=6, chunk_lines=1 << 17, max_chunks=4,
                 chunks_when_interactive=3, window_streams=2, window_blocks_per_sm=0, window_order="srpt"):
        self.fields = dict(fields)
        self.budget = int(hbm_budget)
        self.used = 0
        self.device = torch.device(device)
        self.classes = classes or self.CLASSES
        if max_batch is not None:
            self.classes = tuple((ub, min(int(max_batch), mb), fl) for ub, mb, fl in self.classes)
        # smaller requests get higher stream priority: the block scheduler
        # dispatches their blocks ahead of a large batch's remaining ones
        lo, hi = torch.cuda.Stream.priority_range() if hasattr(torch.cuda.Stream, "priority_range") else (0, -1)
        prios = [max(hi, lo - (len(self.classes) - 1 - c)) for c in range(len(self.classes))]
        prios = [hi if c == 0 else lo for c in range(len(self.classes))] if len(set(prios)) < 2 else prios
        # at least one stream per batch a class may have in flight: batches
        # that shared a stream would run one after another
        self.streams = [[torch.cuda.Stream(device=self.device, priority=prios[c])
                         for _ in range(max(1, streams, int(self.classes[c][2])))]
                        for c in range(len(self.classes))]
        self._next_stream = [0] * len(self.classes)
        self.s_len, self.h_min, self.h_max = s_len, h_min, h_max
        self.tile = tile
        # batches of all but the smallest class keep at most this many of
        # the 8 resident block slots per SM, so the smallest requests' blocks
        # (on the highest-priority stream) start at once (0 = no cap)
        self.big_blocks_per_sm = int(big_blocks_per_sm)
        # main traces of classes > 0 run as windows of chunk_lines lines (a
        # multiple of 32; 0 = one launch per batch)
        self.chunk_lines = (int(chunk_lines) + 31) // 32 * 32
        self.max_chunks, self.chunks_when_interactive = int(max_chunks), int(chunks_when_interactive)
        # windows of one batch alternate over these streams (per class, at the
        # class's priority), so one window's tail overlaps the next window;
        # their blocks are capped at window_blocks_per_sm per SM (0 = none:
        # one line per thread, blocks retire as they finish)
        self.window_streams = [[torch.cuda.Stream(device=self.device, priority=prios[c])
                                for _ in range(max(1, int(window_streams)))] for c in range(len(self.classes))]
        self.window_blocks_per_sm = int(window_blocks_per_sm)
        # order in which batches get their next windows: "srpt" (the batch
        # with the fewest main-trace lines left first, whatever its class;
        # the default: it cut the p99 slowdown at 80 % load from 10.8x to
        # 7.8x isolated on the wide mix) or "class" (smaller class first,
        # then the oldest batch)
        if window_order not in ("class", "srpt"):
            raise ValueError(f"unknown window order {window_order!r}")
        self.window_order = window_order
        self.pending = [collections.deque() for _ in self.classes]
        self.flights = []
        self.done = []
        self.batches = 0

    # ---- request intake ----
    def submit(self, req: QRequest, now=None):
        if req.field not in self.fields:
            raise KeyError(f"unknown field {req.field!r}")
        if req.n0 < 3 or req.n1 < 3:
            raise ValueError("a request needs at least 3 x 3 seeds per plane")
        nb = request_bytes(req)
        if nb > self.budget:
            raise MemoryError(f"request {req.rid} needs {nb} B, more than the HBM budget {self.budget} B")
        req.meta["bytes"] = nb
        req.meta["class"] = next(c for c, (ub, _, _) in enumerate(self.classes) if req.seeds <= ub)
        req.t_submit = time.perf_counter() if now is None else now
        self.pending[req.meta["class"]].append(req)

    # ---- one scheduler turn ----
    def step(self):
        """Retires finished batches, then, per size class, admits waiting
        requests (arrival order, within the HBM budget and the class's batch
        size and in-flight limits) and launches them as one batch on that
        class's streams.  Returns True if anything happened."""
        progressed = self._retire()
        for c, (_, max_batch, max_flights) in enumerate(self.classes):
            q = self.pending[c]
            if not q or sum(1 for fl in self.flights if fl.cls == c) >= max_flights:
                continue
            group, nbytes = [], 0
            while q and len(group) < max_batch:
                r = q[0]
                if self.used + nbytes + r.meta["bytes"] > self.budget:
                    break
                q.popleft()
                group.append(r)
                nbytes += r.meta["bytes"]
            if group:
                self._launch(group, nbytes, c)
                progressed = True
        return self._feed() or progressed

    def _feed(self):
        """Queues main-trace windows of chunked batches, smallest class and
        oldest batch first, while fewer than the allowed number are on the
        device; a batch whose last window is queued gets its post steps."""
        chunked = [fl for fl in self.flights if fl.event is None]
        if not chunked:
            return False
        interactive = any(fl.cls == 0 for fl in self.flights)
        allowed = self.chunks_when_interactive if interactive else self.max_chunks
        busy = sum(fl.windows_in_flight() for fl in chunked)
        progressed = False
        key = (lambda f: f.cls) if self.window_order == "class" else (lambda f: f.lines - f.next_lo)
        for fl in sorted(chunked, key=key):
            wss = self.window_streams[fl.cls]
            while busy < allowed and fl.next_lo < fl.lines:
                hi = min(fl.lines, fl.next_lo + self.chunk_lines)
                k = fl.nwin % len(wss)
                ws = wss[k]
                ws.wait_event(fl.ready)
                with torch.cuda.stream(ws):
                    fl.qb.run_main(stream=ws, lo=fl.next_lo, hi=hi)
                    ev = torch.cuda.Event()
                    ev.record(ws)
                fl.windows.append(ev)
                fl.last[k] = ev
                fl.next_lo, fl.nwin = hi, fl.nwin + 1
                busy += 1
                progressed = True
            if fl.next_lo >= fl.lines:
                self._post(fl)
                progressed = True
        return progressed

    def _post(self, fl):
        """Queues the batch's post-trace steps, the D2H copies of its Q maps
        and its completion event on its stream, after its last windows."""
        for ev in fl.last.values():
            fl.stream.wait_event(ev)
        with torch.cuda.stream(fl.stream):
            qs = fl.qb.run_post(stream=fl.stream)
            # one pinned buffer for the batch's Q maps (each result a view)
            h = torch.empty(sum(q.numel() for q in qs), dtype=torch.float64, pin_memory=True)
            o = 0
            for q in qs:
                hv = h[o:o + q.numel()].view(q.shape)
                hv.copy_(q, non_blocking=True)
                fl.hosts.append(hv)
                o += q.numel()
            fl.event = torch.cuda.Event()
            fl.event.record(fl.stream)

    def _retire(self):
        progressed = False
        keep = []
        for fl in self.flights:
            if fl.event is not None and fl.event.query():
                t = time.perf_counter()
                for r, h in zip(fl.reqs, fl.hosts):
                    r.t_done = t
                    r.result = h.numpy()
                    self.done.append(r)
                self.used -= fl.nbytes
                progressed = True
            else:
                keep.append(fl)
        self.flights = keep
        return progressed

    def _launch(self, group, nbytes, cls):
        st = self.streams[cls][self._next_stream[cls]]
        self._next_stream[cls] = (self._next_stream[cls] + 1) % len(self.streams[cls])
        t = time.perf_counter()
        with torch.cuda.stream(st):
            jobs = []
            for r in group:
                r.t_admit = t
                n, u, v = plane_axes(r.normal)
                prm = absolute_rkf45(tol=r.tol, h_min=self.h_min, h_max=self.h_max)
                jobs.append(dict(field=self.fields[r.field], params=prm, center=r.center, normal=n, u=u, v=v,
                                 spacing=r.spacing, n0=r.n0, n1=r.n1, nplanes=r.nplanes, s_len=self.s_len))
            windowed = cls > 0 and self.chunk_lines > 0
            cap = self.window_blocks_per_sm if windowed else self.big_blocks_per_sm if cls > 0 else 0
            # the native batch: seeds, tile orders, job tables and every
            # launch of the pipeline queued by the C++ library
            qb = api.PlaneQBatch(jobs, device=self.device, tile=self.tile, stream=st, blocks_per_sm=cap)
        self.used += nbytes
        self.batches += 1
        fl = _Flight(group, qb, cls, st, nbytes)
        self.flights.append(fl)
        if windowed:
            fl.lines = qb.main_lines          # windows queued by _feed
            fl.ready = torch.cuda.Event()
            fl.ready.record(st)
        else:
            with torch.cuda.stream(st):
                qb.run_main(stream=st)
            self._post(fl)

    def idle(self):
        return not any(self.pending) and not self.flights

    def drain(self, poll=2e-4):
        while not self.idle():
            if not self.step():
                time.sleep(poll)

    # ---- a timed stream of requests ----
    def run_stream(self, requests, poll=2e-4):
        """Submits each request at its `arrival` time (seconds from now),
        serving continuously; returns the requests in completion order.  The
        cyclic garbage collector is held off while the stream runs (its
        pauses would stall the scheduling loop) and run once at the end."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        gc_on = gc.isenabled()
        gc.disable()
        try:
            t0 = time.perf_counter()
            k = 0
            self.done = []
            while k < len(reqs) or not self.idle():
                now = time.perf_counter()
                while k < len(reqs) and t0 + reqs[k].arrival <= now:
                    self.submit(reqs[k], now=t0 + reqs[k].arrival)
                    k += 1
                if not self.step():
                    nxt = t0 + reqs[k].arrival - time.perf_counter() if k < len(reqs) else poll
                    time.sleep(max(0.0, min(poll, nxt)))
        finally:
            if gc_on:
                gc.enable()
                gc.collect()
        return list(self.done)


def solve_alone(server: QServer, req: QRequest):
    """The isolated solve: the request alone on an otherwise idle server;
    returns (latency in s, Q)."""
    assert server.idle()
    r = QRequest(**{k: getattr(req, k) for k in ("rid", "field", "n0", "n1", "nplanes", "center", "normal",
                                                     "spacing", "tol")})
    server.submit(r)
    server.drain()
    server.done = [d for d in server.done if d is not r]
    return r.latency, r.result


def latency_stats(done, isolated=None):
    """p50/p99 latency (s), throughput (Q-pixels/s over the busy span) and,
    given {rid: isolated latency}, p50/p99 of latency / isolated."""
    lat = np.array([r.latency for r in done])
    span = max(r.t_done for r in done) - min(r.t_submit for r in done)
    out = {"requests": len(done), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
           "qpixels_per_s": float(sum(r.qpixels for r in done) / span)}
    if isolated:
        ratio = np.array([r.latency / isolated[r.rid] for r in done])
        out["p50_over_isolated"] = float(np.percentile(ratio, 50))
        out["p99_over_isolated"] = float(np.percentile(ratio, 99))
    return out


# --------------------------------------------------------------------------
# The serving-stream workload: resident fields and seeded request streams
# --------------------------------------------------------------------------

def make_fields(n_fields=8, shape=(384, 384, 256), layout="h4b", seed=0, device="cuda"):
    """`n_fields` resident stores of point-charge + twisted-tube fields with
    seeded parameters (synthetic.charges_tube)."""
    from . import synthetic as S
    stores = {}
    for k in range(n_fields):
        spec = S.charges_tube(seed * 1000 + k, shape, n_charges=8)
        B = S.make_field(spec, device=device, as_numpy=False)
        stores[f"f{k}"] = api.FieldStore(*B, layout=layout)
        del B
    return stores


def make_requests(fields_shape, names, count, rate, seed=0, seeds_range=(1e4, 4e6), tols=(1e-3, 1e-4, 1e-5),
                  subbox_prob=0.3):
    """`count` requests with Poisson arrivals at `rate` per second (rate
    None: all at t = 0): log-uniform seed counts, a random field, a random
    plane (or, with probability subbox_prob, a stack of 2-8 planes), a random
    tolerance.  The grid spacing keeps every seed inside the box."""
    rng = np.random.default_rng(seed)
    arrivals = np.random.default_rng(seed + 1)  # own stream: same requests at every rate
    nx, ny, nz = fields_shape
    t = 0.0
    out = []
    for k in range(count):
        if rate:
            t += arrivals.exponential(1.0 / rate)
        total = float(np.exp(rng.uniform(np.log(seeds_range[0]), np.log(seeds_range[1]))))
        npl = int(rng.integers(2, 9)) if rng.random() < subbox_prob else 1
        side = max(3, int(round(np.sqrt(total / npl))))
        n0 = max(3, int(round(side * rng.uniform(0.7, 1.3))))
        n1 = max(3, int(round(total / npl / n0)))
        normal = rng.normal(size=3)
        normal /= np.linalg.norm(normal)
        reach = 0.42 * min(nx - 1, ny - 1, nz - 1)
        spacing = min(1.0, reach / (0.5 * np.hypot(n0, n1) + npl))
        center = (0.5 * (nx - 1) + rng.uniform(-0.05, 0.05) * nx, 0.5 * (ny - 1) + rng.uniform(-0.05, 0.05) * ny,
                  0.5 * (nz - 1) + rng.uniform(-0.05, 0.05) * nz)
        out.append(QRequest(rid=k, field=names[int(rng.integers(len(names)))], n0=n0, n1=n1, nplanes=npl,
                            center=center, normal=tuple(normal), spacing=float(spacing),
                            tol=float(tols[int(rng.integers(len(tols)))]), arrival=t))
    return out


# --------------------------------------------------------------------------
# An ideal scheduler on the same request stream: the bound on what any
# scheduler of this server could reach
# --------------------------------------------------------------------------

def fluid_schedule(arrival, work, cap, capacity=1.0, policy="srpt"):
    """Completion times of jobs on a fluid server of `capacity` work units
    per second with free, instant preemption: job i arrives at arrival[i],
    needs work[i] units and runs at most cap[i] units per second (its rate
    when alone).  Policies share the capacity among the jobs present:
    'srpt' (least remaining work first, each up to its cap), 'ps' (equal
    shares, water-filled over the caps) or 'fcfs' (oldest first, up to its
    cap).  Returns an array of completion times."""
    arrival = np.asarray(arrival, float)
    work = np.asarray(work, float)
    cap = np.asarray(cap, float)
    n = len(arrival)
    if policy not in ("srpt", "ps", "fcfs"):
        raise ValueError(f"unknown policy {policy!r}")
    if not (len(work) == len(cap) == n):
        raise ValueError("arrival, work and cap differ in length")
    if np.any(work < 0) or np.any(cap <= 0) or capacity <= 0:
        raise ValueError("work must be >= 0 and caps and capacity > 0")
    if n == 0:
        return np.zeros(0)
    order = np.argsort(arrival, kind="stable")
    rem = work.copy()
    done = np.full(n, np.nan)
    active = []
    nxt = 0
    t = float(arrival[order[0]])
    while nxt < n or active:
        while nxt < n and arrival[order[nxt]] <= t:
            i = int(order[nxt])
            nxt += 1
            if rem[i] <= 0:
                done[i] = arrival[i]
            else:
                active.append(i)
        if not active:
            t = float(arrival[order[nxt]])
            continue
        rate = {}
        if policy == "ps":
            left, pending = capacity, sorted(active, key=lambda j: cap[j])
            while pending:
                share = left / len(pending)
                j = pending[0]
                if cap[j] <= share:
                    rate[j] = cap[j]
                    left -= cap[j]
                    pending.pop(0)
                else:
                    for k in pending:
                        rate[k] = share
                    break
        else:
            key = (lambda j: (rem[j], arrival[j], j)) if policy == "srpt" else (lambda j: (arrival[j], j))
            left = capacity
            for j in sorted(active, key=key):
                rate[j] = min(cap[j], left)
                left -= rate[j]
        dt_done = min((rem[j] / rate[j] for j in active if rate[j] > 0), default=np.inf)
        dt_arr = arrival[order[nxt]] - t if nxt < n else np.inf
        dt = min(dt_done, dt_arr)
        for j in active:
            rem[j] -= rate[j] * dt
        t += dt
        still = []
        for j in active:
            if rem[j] <= 1e-9 * work[j]:  # remaining work within rounding of zero
                done[j] = t
            else:
                still.append(j)
        active = still
    return done


def _deadlines_feasible(arrival, work, cap, deadline, capacity):
    """Whether the fluid server (capacity per second, job i at most cap[i]
    per second, preemption free) can finish every job i between arrival[i]
    and deadline[i]: a transportation problem between jobs and the intervals
    of time their windows share, solved as a maximum flow (source -> job:
    its work; job -> interval inside its window: cap x length; interval ->
    sink: capacity x length).  Amounts are counted in integer units with
    every capacity rounded up and every work rounded down, so the test can
    only err towards feasible (a bound built on it stays a lower bound)."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import maximum_flow
    n = len(arrival)
    pts = np.unique(np.concatenate([arrival, deadline]))
    lo, hi = pts[:-1], pts[1:]
    length = hi - lo
    m = len(length)
    # integer unit: the total work spread over ~2^30 units
    unit = max(float(work.sum()), 1e-300) / float(1 << 30)
    src, snk = 0, 1 + n + m
    rows, cols, caps = [], [], []
    for i in range(n):
        k0 = int(np.searchsorted(pts, arrival[i], side="left"))
        k1 = int(np.searchsorted(pts, deadline[i], side="left"))
        if k1 <= k0:
            continue
        ks = np.arange(k0, k1)
        rows.append(np.full(len(ks), 1 + i))
        cols.append(1 + n + ks)
        caps.append(np.ceil(cap[i] * length[ks] / unit))
    rows.append(np.zeros(n, np.int64))
    cols.append(1 + np.arange(n))
    need = np.floor(work / unit)
    caps.append(need)
    rows.append(1 + n + np.arange(m))
    cols.append(np.full(m, snk))
    caps.append(np.ceil(capacity * length / unit))
    r, c, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(caps)
    v = np.minimum(v, 2**31 - 1).astype(np.int32)
    g = csr_matrix((v, (r.astype(np.int32), c.astype(np.int32))), shape=(snk + 1, snk + 1))
    g.sum_duplicates()
    return maximum_flow(g, src, snk).flow_value >= int(need.sum())


def min_max_stretch(arrival, work, cap, isolated, capacity=1.0, rel=1e-3):
    """A lower bound, within `rel`, on the largest ratio of response time to
    isolated time that any schedule of the jobs on the fluid server reaches
    (fluid_schedule's model): the smallest s for which every job i can
    finish by arrival[i] + s * isolated[i] (bisection on s over the
    feasibility test; s >= 1, and no schedule beats s by more than `rel`).
    Minimising the largest ratio is not what SRPT does (it minimises the
    mean response time), so this is the floor for a worst-request figure."""
    arrival = np.asarray(arrival, float)
    work = np.asarray(work, float)
    cap = np.asarray(cap, float)
    iso = np.asarray(isolated, float)
    if len(arrival) == 0:
        return 1.0
    hi = max(1.0, float(np.max((fluid_schedule(arrival, work, cap, capacity, "srpt") - arrival) / iso)))
    lo = 1.0
    if _deadlines_feasible(arrival, work, cap, arrival + lo * iso, capacity):
        return lo
    while hi - lo > rel * lo:
        mid = 0.5 * (lo + hi)
        if _deadlines_feasible(arrival, work, cap, arrival + mid * iso, capacity):
            hi = mid
        else:
            lo = mid
    return lo


def ideal_bound(requests, isolated, saturated_span, policies=("srpt", "ps"), min_max=False):
    """p50/p99 of latency / isolated solve that an ideal fluid scheduler
    (free preemption, perfect sharing of the GPU) reaches on `requests`
    under each policy, and with `min_max` the smallest worst-request ratio
    any schedule reaches (min_max_stretch).

    A request's work is its Q-pixels times the GPU time per Q-pixel of the
    most efficient isolated solve at its tolerance (the largest requests fill
    the GPU, so theirs is the full-GPU cost); its rate when alone is
    work / isolated (small requests cannot fill the GPU).  The capacity is
    the work of the whole set over the span the server took to finish it
    when all were submitted at once, so the offered load of the stream is
    the same fraction of capacity as the measured stream's."""
    tpx = {}
    for r in requests:
        c = isolated[r.rid] / r.qpixels
        tpx[r.tol] = min(tpx.get(r.tol, np.inf), c)
    work = np.array([r.qpixels * tpx[r.tol] for r in requests])
    iso = np.array([isolated[r.rid] for r in requests])
    cap = work / iso
    capacity = work.sum() / saturated_span
    arrival = np.array([r.arrival for r in requests])
    out = {}
    for pol in policies:
        ratio = (fluid_schedule(arrival, work, cap, capacity, pol) - arrival) / iso
        out[pol] = [float(np.percentile(ratio, 50)), float(np.percentile(ratio, 99))]
    if min_max:
        out["min_max"] = min_max_stretch(arrival, work, cap, iso, capacity)
    return out


def sweep(server: QServer, fields_shape, count=512, fractions=(0.5, 0.8), seed=7, seeds_range=(1e4, 4e6),
          batched_server: QServer | None = None, keep_alone=8, alone_out: dict | None = None):
    """Isolated solve of every request, the saturated throughput (all
    requests at once), then Poisson streams at fractions of the saturated
    request rate.  With `batched_server` (e.g. one launching whole batches,
    chunk_lines=0) the saturated rate the fractions refer to is that
    server's, and `server`'s own saturated throughput is reported beside it.
    Returns a dict of latency_stats per point, each with the ideal fluid
    scheduler's figures on the same stream built from the measured isolated
    solves (SRPT and processor-sharing p50/p99, and the smallest worst-request
    ratio any schedule reaches) beside this server's worst ratio.  The first
    `keep_alone` requests' isolated results are compared with their results
    in every stream ('alone_vs_mix_identical', bit for bit, NaN where NaN);
    with `alone_out` they are also returned there ({rid: (request, Q)})."""
    names = sorted(server.fields)
    burst = make_requests(fields_shape, names, count, None, seed=seed, seeds_range=seeds_range)
    iso, alone = {}, {}
    for r in burst:
        iso[r.rid], q = solve_alone(server, r)
        if r.rid < keep_alone:
            alone[r.rid] = q
            if alone_out is not None:
                alone_out[r.rid] = (r, q)

    def same_as_alone(done):
        hit = [r for r in done if r.rid in alone]
        ok = sum(1 for r in hit if np.array_equal(r.result, alone[r.rid], equal_nan=True))
        return f"{ok}/{len(hit)}"
    done = (batched_server or server).run_stream(burst)
    sat = dict(latency_stats(done, iso), alone_vs_mix_identical=same_as_alone(done))
    span = max(r.t_done for r in done) - min(r.t_submit for r in done)
    sat_rate = count / span
    res = {"saturated": sat, "isolated_p50_s": float(np.median(list(iso.values())))}
    if batched_server is not None:
        own = make_requests(fields_shape, names, count, None, seed=seed, seeds_range=seeds_range)
        res["saturated_this_server"] = latency_stats(server.run_stream(own), iso)
    for f in fractions:
        reqs = make_requests(fields_shape, names, count, f * sat_rate, seed=seed, seeds_range=seeds_range)
        done = server.run_stream(reqs)
        st = dict(latency_stats(done, iso), offered_req_per_s=f * sat_rate)
        # what an ideal fluid scheduler reaches on the same stream: [p50, p99]
        ideal = ideal_bound(reqs, iso, span, min_max=True)
        st["ideal_min_max_over_isolated"] = ideal.pop("min_max")
        st["ideal_fluid_p50_p99_over_isolated"] = ideal
        st["max_over_isolated"] = float(max(r.latency / iso[r.rid] for r in done))
        st["alone_vs_mix_identical"] = same_as_alone(done)
        for c in range(len(server.classes)):
            rr = [r.latency / iso[r.rid] for r in done if r.meta["class"] == c]
            if rr:
                st[f"class{c}_p50_p90_over_isolated"] = [float(np.percentile(rr, 50)), float(np.percentile(rr, 90))]
        res[f"rate_{f:.2f}"] = st
    return res
