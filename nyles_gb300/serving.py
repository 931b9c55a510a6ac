"""Serving engine: continuous batching of independent Nyles runs on one GPU.

Requests (a lock exchange or a Taylor-Green case on an n^3 grid, a number of steps, a
noise seed) arrive over time. Runs of the same case and grid form a bucket: its runs
live in the slots of one device buffer, and one batched CUDA graph of k time steps,
whose every kernel covers all slots of the bucket, advances all of them with a single
launch (nyles_model_batch_capture). A request is admitted as soon as its bucket has a
free slot (or a new bucket fits the HBM budget); it joins the bucket's next launch
after its initial projection, and frees its slot when its last launch completes.
Buckets run on their own streams, so every size overlaps on the device.
Completion latency = time from arrival to the end of the run's last step.

The reference has no serving layer (one experiment per process, core/nyles.py).
"""
import functools
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from . import parameters
from .nyles import Nyles

TWO_PI = 6.283185307179586

# Cases of the ensemble. The lock exchange uses a unit cube: with cubic cells the
# reference's projection is exact (an anisotropic box makes it unstable).
CASES = {
    "lock": dict(geometry="closed", L=(1.0, 1.0, 1.0), dt=2e-3),
    "tgv": dict(geometry="perio_xyz", L=(TWO_PI, TWO_PI, TWO_PI), dt=5e-3),
}


@dataclass
class Request:
    rid: int
    case: str
    n: int
    seed: int
    steps: int
    arrival: float          # seconds after the start of the stream

    @property
    def bucket(self):
        return (self.case, self.n)


@dataclass
class Result:
    rid: int
    case: str
    n: int
    steps: int
    arrival: float
    admitted: float
    done: float
    cells: int
    mg_vcycles: int = 0
    # "ok"; "refused" (footprint above the whole budget, never admitted); "blowup" (a
    # non-finite velocity or pressure solve); "not_converged" (finished, but some
    # pressure solve stopped at mg_maxite above the tolerance)
    status: str = "ok"

    @property
    def latency(self):
        return self.done - self.arrival

    @property
    def completed(self):
        return self.status in ("ok", "not_converged")


def make_requests(count=96, rate=20.0, seed=5, steps=300, sizes=(32, 48, 64, 96, 128)):
    """Seeded Poisson stream: exponential inter-arrival times at `rate` per second, case
    and size uniform, a per-run noise seed drawn from the same generator."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        case = ("lock", "tgv")[int(rng.integers(2))]
        n = int(sizes[int(rng.integers(len(sizes)))])
        out.append(Request(i, case, n, int(rng.integers(2 ** 31)), steps, t))
    return out


def build_params(case, n, precision="mixed", mg_tol=1e-6):
    c = CASES[case]
    parameters.InextensibleDict.unfreeze()
    p = parameters.UserParameters()
    p.model["modelname"] = "LES"
    p.model["geometry"] = c["geometry"]
    p.model["Lx"], p.model["Ly"], p.model["Lz"] = c["L"]
    p.time["timestepping"] = "RK3_SSP"
    p.time["auto_dt"] = False
    p.time["dt"] = c["dt"]
    p.discretization["global_nx"] = n
    p.discretization["global_ny"] = n
    p.discretization["global_nz"] = n
    p.gpu["precision"] = precision
    p.gpu["mg_tol"] = mg_tol
    p.gpu["history"] = False
    return p


@functools.lru_cache(maxsize=64)
def case_grid(case, n):
    """The grid of a case on n^3 cells (the coordinates that initial_fields reads)"""
    from . import grid as grid_module
    from .nyles import prepare_parameters
    return grid_module.Grid(prepare_parameters(build_params(case, n)))


def initial_fields(nyl, case, seed):
    """Seeded initial fields (numpy, the (z, y, x) arrays of view('i')): lock exchange
    (b = -0.5 | +0.5 across x = L/2 plus uniform noise 1e-3) or Taylor-Green (u = sin x
    cos y cos z, v = -cos x sin y cos z plus Gaussian noise 1e-4, covariant: times the
    spacing). `nyl`: a Nyles of the case, or its grid."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = getattr(nyl, "grid", nyl)
    if case == "lock":
        xb = g.x_b.view("i").numpy()
        return {"b": np.where(xb < 0.5 * g.Lx, -0.5, 0.5) + 1e-3 * rng.uniform(-1, 1, size=xb.shape)}
    xu, yu, zu = (g.x_vel["i"].view("i").numpy(), g.y_vel["i"].view("i").numpy(), g.z_vel["i"].view("i").numpy())
    xv, yv, zv = (g.x_vel["j"].view("i").numpy(), g.y_vel["j"].view("i").numpy(), g.z_vel["j"].view("i").numpy())
    shape = xu.shape
    u = (np.sin(xu) * np.cos(yu) * np.cos(zu) + 1e-4 * rng.standard_normal(shape)) * g.dx
    v = (-np.cos(xv) * np.sin(yv) * np.cos(zv) + 1e-4 * rng.standard_normal(shape)) * g.dy
    w = 1e-4 * rng.standard_normal(shape) * g.dz
    return {"u_i": u, "u_j": v, "u_k": w}


def initial_state(nyl, case, seed):
    """Write the seeded initial fields of `initial_fields` through view('i')."""
    st = nyl.model.state
    for name, arr in initial_fields(nyl, case, seed).items():
        st.get(name).view("i")[...] = torch.from_numpy(arr)


def footprint_bytes(case, n, precision="mixed", mg_tol=1e-6):
    """Device bytes of one run: 14 state fields, 3 x 4 time-scheme registers, and the
    multigrid workspace (x, b, y per level; in mixed precision also the float-pair
    solution of level 1, or at Krylov tolerances one per RK3 stage and two before each
    for the extrapolated warm start, its float-pair rhs and the two float vectors
    of the Krylov solver), plus 3% and 256 KiB for partial sums, scalars and allocator
    rounding."""
    per = CASES[case]["geometry"]
    e = 8 if precision == "fp64" else 4
    dims = [n + (6 if ax in per else 0) for ax in ("z", "y", "x")]
    vol = dims[0] * dims[1] * dims[2]
    fields = (14 + 3 * 4) * vol * e
    mg, x, z = 0, n, n
    while True:
        mg += 3 * e * z * x * x
        if x == 2 or x % 2 or x < 4:
            break
        x //= 2
        z //= 2
    if precision == "mixed":
        from .model_les import KRYLOV_AUTO_TOL
        pairs = 3 * 3 if mg_tol <= KRYLOV_AUTO_TOL else 1
        mg += (pairs + 1) * 8 * n ** 3 + 2 * 4 * n ** 3
    return int(1.03 * (fields + mg)) + (1 << 18)


# cells that the batched launches of one bucket cover at most (capacity "auto"): a run of
# 128^3 cells fills the device alone, so its bucket batches few runs, while runs of 32^3
# to 64^3 are bound by launch latency and batch up to NYLES_BATCH_RUNS
CELLS_PER_BUCKET = 1 << 23


def auto_capacity(n, cap_max=32):
    """slots of a bucket of n^3-cell runs under capacity 'auto'"""
    return max(1, min(cap_max, CELLS_PER_BUCKET // n ** 3))


# cell-steps one graph launch of a run covers at least (up to GRAPH_KMAX steps): small
# grids take longer graphs, so that each launch keeps the device busy for about as long
# as a 128^3 run's 10 steps and the run does not wait on the host loop between launches
GRAPH_CELL_STEPS = 10 << 21
GRAPH_KMAX = 60


def graph_steps(n, steps):
    """steps per graph launch of an n^3 run of `steps` steps"""
    return steps_per_graph(steps, max(10, min(GRAPH_KMAX, GRAPH_CELL_STEPS // n ** 3)))


def steps_per_graph(steps, kmax=10):
    """largest divisor of `steps` not above kmax: graph launches land exactly on `steps`"""
    for k in range(min(kmax, steps), 0, -1):
        if steps % k == 0:
            return k
    return 1


class Slot:
    """One place of a bucket: a model whose arrays are carved from the slot's part of
    the bucket buffer, and the request it currently serves (None: free). The model is
    built when the slot is first used (`make` returns it): the batched graphs address
    every slot through slot 0's model and the slot's byte offset."""

    def __init__(self, index, make):
        self.index = index
        self._make = make
        self._nyl = None
        self.req = None
        self.projected = False     # the initial projection has been launched
        self.launched = 0
        self.last_event = None     # event of the latest launch that advanced this run
        self.admitted = 0.0
        self.staging = None        # pinned host copies of the initial state, kept until used

    @property
    def nyl(self):
        if self._nyl is None:
            self._nyl = self._make()
        return self._nyl

    @property
    def active(self):
        return self.req is not None and self.projected and self.launched < self.req.steps

    def finished(self):
        if self.req is None or not self.projected:
            return False
        return self.launched >= self.req.steps and (self.last_event is None or self.last_event.query())


class Bucket:
    """The resident runs of one (case, grid, steps per launch) on `capacity` slots of one
    device buffer. Every slot's model is built in an Arena of the same size, so its
    arrays sit at the same offsets: slot r's memory is slot 0's shifted by r x slot_bytes.
    Batched one-step graphs recorded on slot 0's model (nyles_model_batch_capture), one
    per batch size (powers of two up to the capacity, recorded when first needed), advance
    a list of runs, each launch replaying the step graph k times (a k-step graph costs
    more than k times as much host time to record): the table of a launch lists the
    slots' offsets first, so a launch
    covers only as many slots as it advances, and the runs are processed in the smallest
    batch size that holds them. Each run's pressure solves stop on their own, so its
    result is the same whatever else shares the launch. A new run's slot is zeroed, its
    initial state copied from pinned host memory and its initial projection recorded as
    a batched graph too, all queued on the bucket's stream: admission never waits for
    the device."""

    def __init__(self, key, precision, mg_tol, device, capacity, priority=0):
        import ctypes
        from . import _native as nat
        from .nyles import arena_bytes
        from .variables import Arena
        case, n, k = key
        self.key, self.case, self.n, self.k = key, case, n, k
        self.capacity = capacity
        self.slot_bytes = Arena.aligned(arena_bytes(build_params(case, n, precision, mg_tol)))
        self.bytes = self.slot_bytes * capacity
        self.buf = torch.zeros(self.bytes, dtype=torch.uint8, device=device)
        def make(r):
            arena = Arena(self.buf[r * self.slot_bytes:(r + 1) * self.slot_bytes])
            return Nyles(build_params(case, n, precision, mg_tol), device=device, arena=arena)

        self.slots = [Slot(r, functools.partial(make, r)) for r in range(capacity)]
        self.lib = nat.lib()
        self.nat = nat
        tb = ctypes.sizeof(nat.NylesBatchTable)
        self.table = torch.zeros(tb, dtype=torch.uint8, device=device)
        # the host writes delta and active (the leading fields); live and loop_iterations
        # belong to the device
        self.host_bytes = nat.NylesBatchTable.live.offset
        self.ring = [torch.zeros(tb, dtype=torch.uint8).pin_memory() for _ in range(8)]
        self.ring_events = [None] * len(self.ring)
        self.ring_pos = 0
        self.stream = torch.cuda.Stream(device=device, priority=priority)
        self.read_stream = torch.cuda.Stream(device=device, priority=priority)
        self.inflight = []
        self.launches = 0
        self.template = self.slots[0].nyl.model
        self.graphs = {}          # (kind, batch size) -> NylesBatchGraph handle
        self.dt = CASES[case]["dt"]

    # ---- graphs
    def sizes(self):
        out, b = [], 1
        while b < self.capacity:
            out.append(b)
            b *= 2
        return out + [self.capacity]

    def graph(self, kind, nact):
        import ctypes
        size = next(b for b in self.sizes() if b >= nact)
        g = self.graphs.get((kind, size))
        if g is None:
            h = ctypes.c_void_p()
            steps = 1 if kind == "step" else 0      # one step, launched k times
            self.nat.check(self.lib.nyles_model_batch_capture(self.template._h, self.dt, steps, size,
                                                              ctypes.c_void_p(self.table.data_ptr()),
                                                              ctypes.byref(h)))
            g = self.graphs[(kind, size)] = h
        return g, size

    # ---- slots
    def free_slot(self):
        return next((sl for sl in self.slots if sl.req is None), None)

    def resident(self):
        return [sl for sl in self.slots if sl.req is not None]

    def admit(self, slot, req, now, staged=None):
        """Queue on the bucket stream: zero the slot (a fresh allocation's contents) and
        copy the request's initial state in from pinned host memory (`staged`, from
        stage_initial_state, or made here); the projection follows in the next launch
        (`launch`)."""
        slot.req, slot.launched, slot.last_event, slot.projected = req, 0, None, False
        slot.admitted = now
        if staged is None:
            staged = stage_initial_state(req, self.template.dtype)
        lo = slot.index * self.slot_bytes
        with torch.cuda.stream(self.stream):
            self.buf[lo:lo + self.slot_bytes].zero_()
            st = slot.nyl.model.state
            for name, h in staged.items():
                st.get(name).view("i").copy_(h, non_blocking=True)
        slot.staging = staged

    # ---- launches
    def poll(self):
        while self.inflight and self.inflight[0].query():
            self.inflight.pop(0)
        return len(self.inflight)

    def _launch(self, kind, slots):
        g, size = self.graph(kind, len(slots))
        i = self.ring_pos
        self.ring_pos = (i + 1) % len(self.ring)
        if self.ring_events[i] is not None:
            self.ring_events[i].synchronize()          # the pinned buffer's previous copy is done
        t = self.nat.NylesBatchTable.from_address(self.ring[i].data_ptr())
        for r in range(size):
            t.active[r] = 1 if r < len(slots) else 0
            t.delta[r] = slots[r].index * self.slot_bytes if r < len(slots) else 0
        with torch.cuda.stream(self.stream):
            self.table[:self.host_bytes].copy_(self.ring[i][:self.host_bytes], non_blocking=True)
        ev_tab = torch.cuda.Event()
        ev_tab.record(self.stream)
        self.ring_events[i] = ev_tab
        sp = self.nat.stream_ptr(self.stream)
        for _ in range(self.k if kind == "step" else 1):
            self.nat.check(self.lib.nyles_batch_launch(g, sp))
        self.launches += 1

    def launch(self):
        """Project the newly admitted runs, then advance every active run by k steps,
        each group with one graph launch; returns False when there was nothing to do."""
        new = [sl for sl in self.slots if sl.req is not None and not sl.projected]
        if new:
            self._launch("diag", new)
            for sl in new:
                sl.projected = True
        act = [sl for sl in self.slots if sl.active]
        if act:
            self._launch("step", act)
            for sl in act:
                sl.launched += self.k
        if not (new or act):
            return False
        ev = torch.cuda.Event()
        ev.record(self.stream)
        self.inflight.append(ev)
        for sl in new + act:
            sl.last_event = ev
        return True

    # ---- completion
    def outcome(self, slot, keep_state=False):
        """(status, V-cycles, final fields or None) of a finished run, read on the read
        stream once its last launch is complete: "blowup" when a pressure solve met a
        non-finite norm (a non-finite velocity reaches every projection), "not_converged"
        when a solve stopped at maxite above the tolerance, else "ok"."""
        import ctypes
        nat = self.nat
        m = slot.nyl.model
        st = nat.NylesMgStats()
        with torch.cuda.stream(self.read_stream):
            if slot.last_event is not None:
                self.read_stream.wait_event(slot.last_event)
            nat.check(self.lib.nyles_model_device_stats(m._h, ctypes.byref(st), nat.stream_ptr(self.read_stream)))
            status = "blowup" if st.nonfinite > 0 else ("not_converged" if st.not_converged > 0 else "ok")
            fields = None
            if keep_state:
                fields = {s: m.state.get(s).view("i").double().cpu().numpy() for s in ("b", "u_i", "u_j", "u_k", "p")}
        return status, st.vcycles, fields

    def release(self, slot):
        slot.req = None
        slot.last_event = None
        slot.staging = None

    def loop_iterations(self):
        """multigrid loop-body iterations the batched launches ran (device counter)"""
        import ctypes
        t = self.nat.NylesBatchTable()
        host = self.table.cpu()
        ctypes.memmove(ctypes.addressof(t), host.data_ptr(), ctypes.sizeof(t))
        return t.loop_iterations

    def close(self):
        """Count the loop kernels, release the graphs and the memory."""
        self.stream.synchronize()
        if self.graphs:
            g = next(iter(self.graphs.values()))
            self.nat.check(self.lib.nyles_batch_note_iterations(g, self.loop_iterations()))
        for g in self.graphs.values():
            self.lib.nyles_batch_destroy(g)
        self.graphs = {}
        self.slots = []
        self.template = None
        self.buf = None


def stage_initial_state(req, dtype, grid=None):
    """{field: pinned host tensor} of a request's initial state in the model's dtype
    (host work only: the engine runs it on worker threads ahead of admission, with the
    grid built beforehand on the engine's thread, which alone touches the parameters)"""
    fields = initial_fields(grid if grid is not None else case_grid(req.case, req.n), req.case, req.seed)
    return {name: torch.from_numpy(arr).to(dtype).pin_memory() for name, arr in fields.items()}


def remaining_work(bucket):
    """cells x steps not yet launched in a bucket"""
    return sum(bucket.n ** 3 * max(0, sl.req.steps - sl.launched) for sl in bucket.slots if sl.req is not None)


class ServingEngine:
    """Continuous batching: admission against an HBM budget, resident runs grouped into
    size buckets, one batched graph launch per bucket advancing all of its runs.

    A request is admitted as soon as its bucket (case, grid and steps per launch) has a
    free slot, or a new bucket fits the budget; a request larger than the whole budget
    is refused at once. Each bucket keeps up to `inflight` launches queued on its own
    stream (CUDA priority by the per-run work n^3 x steps, smallest first, with
    priority "work"; equal with "none"), so buckets of every size overlap on the device.
    `capacity` = slots per bucket (at most NYLES_BATCH_RUNS), or "auto": as many runs as
    CELLS_PER_BUCKET cells hold (auto_capacity). A bucket whose runs have all finished
    stays, idle, with its models and graphs for later requests of the same key; idle
    buckets give their memory back, least recently used first, when a new bucket needs
    it, and all are released when serve returns. The initial states of queued requests
    are built on `prep_threads` host threads while the loop keeps launching. `window` =
    W launches only the W buckets with the least
    remaining work (cells x steps not yet launched) at each tick, so that small runs
    finish soon after they arrive and the large ones, which set the makespan, fill the
    device afterwards; None launches every bucket. Completion latency = arrival to the
    end of the run's last launch."""

    def __init__(self, hbm_budget_bytes=120e9, precision="mixed", mg_tol=1e-6, device=None, inflight=2,
                 clock=time.perf_counter, bucket_factory=None, priority="work", capacity="auto", window=None,
                 prep_threads=4, prep_ahead=16):
        if window is not None and window < 1:
            raise ValueError("window must be None or >= 1")
        self.window = window
        if priority not in ("work", "none"):
            raise ValueError("priority must be 'work' or 'none'")
        if capacity != "auto" and not 1 <= capacity <= 32:
            raise ValueError("capacity must be 'auto' or 1..32 (NYLES_BATCH_RUNS)")
        self.prep_threads = prep_threads
        self.prep_ahead = prep_ahead
        self.priority = priority
        self.capacity = capacity
        self.budget = float(hbm_budget_bytes)
        self.precision = precision
        self.mg_tol = mg_tol
        self.bucket_factory = bucket_factory or Bucket
        if device is None and bucket_factory is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device) if device is not None else None
        self.inflight = inflight
        self.clock = clock
        self.used = 0
        self.peak_used = 0
        self.max_active = 0
        self.buckets_made = 0
        self.launches = 0

    def capacity_for(self, n):
        return auto_capacity(n) if self.capacity == "auto" else self.capacity

    def serve(self, requests, realtime=True, keep_states=False):
        """Serve `requests` (arrival times relative to now when `realtime`, else all at
        once). Returns (results, final_states) with final_states[rid] = dict of numpy
        prognostic fields when keep_states."""
        pending = sorted(requests, key=lambda r: r.arrival)
        prio = self.stream_priorities(requests)
        queue, buckets, results, states = [], {}, [], {}
        # initial states built on host threads ahead of admission (real device only)
        pool = (ThreadPoolExecutor(self.prep_threads) if self.prep_threads > 0 and self.device is not None
                and self.device.type == "cuda" else None)
        dtype = torch.float64 if self.precision == "fp64" else torch.float32
        staging = {}
        self._idle = {}           # bucket key -> time its last run left (idle buckets)
        t0 = self.clock()
        nxt = 0
        try:
            while nxt < len(pending) or queue or any(b.resident() for b in buckets.values()):
                nxt, queue = self._tick(pending, nxt, queue, buckets, results, states, prio, realtime,
                                        keep_states, t0, pool, staging, dtype)
        finally:
            for key in list(buckets):
                self._release(buckets, key)
            if pool is not None:
                pool.shutdown(wait=True, cancel_futures=True)
        if self.device is not None and self.device.type == "cuda":
            torch.cuda.synchronize(self.device)
        return sorted(results, key=lambda r: r.rid), states

    def _tick(self, pending, nxt, queue, buckets, results, states, prio, realtime, keep_states, t0, pool,
              staging, dtype):
        """one pass of the serving loop: arrivals, admission, launches, completions"""
        now = self.clock() - t0
        while nxt < len(pending) and (not realtime or pending[nxt].arrival <= now):
            queue.append(pending[nxt])
            nxt += 1
        if pool is not None:
            for req in queue[:self.prep_ahead]:
                if req.rid not in staging and footprint_bytes(req.case, req.n, self.precision, self.mg_tol) <= self.budget:
                    staging[req.rid] = pool.submit(stage_initial_state, req, dtype, case_grid(req.case, req.n))
        # admission, in arrival order; a request whose bucket is full, or whose
        # initial state is still being built, waits without blocking the others
        waiting = []
        for req in queue:
            need = footprint_bytes(req.case, req.n, self.precision, self.mg_tol)
            if need > self.budget:
                results.append(Result(req.rid, req.case, req.n, req.steps, req.arrival if realtime else 0.0,
                                      now, now, req.n ** 3, 0, "refused"))
                continue
            fut = staging.get(req.rid)
            if fut is not None and not fut.done():
                waiting.append(req)
                continue
            key = (req.case, req.n, graph_steps(req.n, req.steps))
            b = buckets.get(key)
            if b is None:
                want = self.capacity_for(req.n)
                # buckets left idle by earlier runs give their memory back, least recently
                # used first, when a new bucket needs it
                idle = sorted((k for k in buckets if k in self._idle), key=lambda k: self._idle[k])
                while idle and self.used + want * need > self.budget:
                    self._release(buckets, idle.pop(0))
                cap = min(want, int((self.budget - self.used) // need))
                if cap < 1:
                    waiting.append(req)
                    continue
                b = self.bucket_factory(key, self.precision, self.mg_tol, self.device, cap,
                                        priority=prio[req.rid])
                buckets[key] = b
                self.buckets_made += 1
                self.used += b.bytes
                self.peak_used = max(self.peak_used, self.used)
            slot = b.free_slot()
            if slot is None:
                waiting.append(req)
                continue
            fut = staging.pop(req.rid, None)
            b.admit(slot, req, self.clock() - t0, staged=fut.result() if fut is not None else None)
        queue = waiting
        self.max_active = max(self.max_active, sum(len(b.resident()) for b in buckets.values()))
        # launches: every bucket, or the `window` with the least remaining work
        busy = False
        order = list(buckets.values())
        if self.window is not None:
            order = sorted(order, key=remaining_work)[:self.window]
        for b in order:
            if b.poll() < self.inflight:
                busy |= b.launch()
        # completion
        for key in list(buckets):
            b = buckets[key]
            for sl in b.slots:
                if sl.finished():
                    req = sl.req
                    status, vcycles, fields = b.outcome(sl, keep_states)
                    done = self.clock() - t0
                    results.append(Result(req.rid, req.case, req.n, req.steps, req.arrival if realtime else 0.0,
                                          sl.admitted, done, req.n ** 3, vcycles, status))
                    if keep_states and fields is not None:
                        states[req.rid] = fields
                    b.release(sl)
            if b.resident():
                self._idle.pop(key, None)
            else:
                self._idle.setdefault(key, self.clock() - t0)
        if not busy:
            if any(b.resident() for b in buckets.values()) or staging:
                time.sleep(2e-4)
            elif not queue and nxt < len(pending):
                time.sleep(max(0.0, min(2e-3, pending[nxt].arrival - (self.clock() - t0))))
        return nxt, queue

    def _release(self, buckets, key):
        b = buckets.pop(key)
        self._idle.pop(key, None)
        self.launches += b.launches
        b.close()
        self.used -= b.bytes

    def stream_priorities(self, requests, levels=None):
        """{rid: stream priority}: the distinct work values (n^3 x steps) of the requests,
        smallest first, spread over the device's priority range (greatest priority to
        the least work); 0 for all with priority "none"."""
        if self.priority == "none" or not requests:
            return {r.rid: 0 for r in requests}
        if levels is None:
            least, greatest = (torch.cuda.Stream.priority_range() if self.device is not None
                               and self.device.type == "cuda" else (0, 0))
        else:
            least, greatest = levels
        nlev = least - greatest + 1
        works = sorted({r.n ** 3 * r.steps for r in requests})
        rank = {w: i for i, w in enumerate(works)}
        return {r.rid: greatest + min(nlev - 1, rank[r.n ** 3 * r.steps] * nlev // len(works)) for r in requests}


def run_sequential(requests, precision="fp64", mg_tol=1e-6, device=None, keep_states=False):
    """Baseline: the same runs one at a time through model.forward (by default FP64),
    in arrival order; a run starts at max(arrival, end of the previous run)."""
    results, states = [], {}
    clock = 0.0
    for req in sorted(requests, key=lambda r: r.arrival):
        nyl = Nyles(build_params(req.case, req.n, precision, mg_tol), device=device)
        initial_state(nyl, req.case, req.seed)
        torch.cuda.synchronize()
        t = time.perf_counter()
        m = nyl.model
        m.diagnose_var(m.state)
        dt = CASES[req.case]["dt"]
        for _ in range(req.steps):
            m.forward(0.0, dt)
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        start = max(clock, req.arrival)
        clock = start + el
        results.append(Result(req.rid, req.case, req.n, req.steps, req.arrival, start, clock, req.n ** 3,
                              m.mg_stats()["vcycles"]))
        if keep_states:
            states[req.rid] = {s: m.state.get(s).view("i").double().cpu().numpy()
                               for s in ("b", "u_i", "u_j", "u_k", "p")}
        del nyl, m
    return results, states


def sequential_estimate(requests, precision="fp64", mg_tol=1e-6, device=None, sample_steps=10, warmup=2):
    """The baseline of run_sequential without running every step: for each bucket (case,
    grid) of the requests, the setup (model build, initial projection) and `sample_steps`
    eager steps after `warmup` are timed once; the arrival queue is then replayed with
    duration = setup + steps x step time per run, one run at a time. Returns (results,
    {bucket: {"setup_s", "step_s"}})."""
    timing = {}
    for case, n in sorted({r.bucket for r in requests}):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nyl = Nyles(build_params(case, n, precision, mg_tol), device=device)
        initial_state(nyl, case, 0)
        m = nyl.model
        m.diagnose_var(m.state)
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        dt = CASES[case]["dt"]
        for _ in range(warmup):
            m.forward(0.0, dt)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(sample_steps):
            m.forward(0.0, dt)
        torch.cuda.synchronize()
        timing[(case, n)] = {"setup_s": setup, "step_s": (time.perf_counter() - t0) / sample_steps}
        del nyl, m
    return replay_queue(requests, lambda r: timing[r.bucket]["setup_s"] + r.steps * timing[r.bucket]["step_s"]), timing


def replay_queue(requests, duration):
    """One run at a time in arrival order: a run starts at max(arrival, end of the
    previous run) and lasts duration(request) seconds."""
    results, clock = [], 0.0
    for req in sorted(requests, key=lambda r: r.arrival):
        start = max(clock, req.arrival)
        clock = start + duration(req)
        results.append(Result(req.rid, req.case, req.n, req.steps, req.arrival, start, clock, req.n ** 3))
    return results


def summarize(results, makespan=None):
    """Latency percentiles and throughput over the completed runs (status "ok" or
    "not_converged"); refused and blown-up runs are counted, not timed."""
    done = [r for r in results if r.completed]
    counts = {k: sum(1 for r in results if r.status == k) for k in ("refused", "blowup", "not_converged")}
    if not done:
        return dict(runs=0, **counts)
    lat = np.array([r.latency for r in done])
    cells = sum(r.cells * r.steps for r in done)
    span = makespan if makespan is not None else (max(r.done for r in done) - min(r.arrival for r in done))
    return dict({"runs": len(done), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                 "mean_s": float(lat.mean()), "makespan_s": float(span), "cell_steps_per_s": cells / span}, **counts)
