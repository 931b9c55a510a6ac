"""Serving engine: continuous batching of independent Nyles runs on one GPU.

Requests (a lock exchange or a Taylor-Green case on an n^3 grid, a number of steps, a
noise seed) arrive over time. The engine admits a request as soon as its device
footprint fits the HBM budget, builds the run (state, multigrid, initial projection)
and captures a CUDA graph of k time steps; from then on the run is resident and is
advanced by replaying that graph on its own stream. Every engine tick keeps up to two
graph launches in flight per run, so runs of every size overlap on the device while new
ones are admitted and finished ones release their memory. Runs are grouped into size
buckets (same case and grid: same graph shape and footprint) for admission and
reporting. Completion latency = time from arrival to the end of the run's last step.

The reference has no serving layer (one experiment per process, core/nyles.py).
"""
import time
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


def initial_state(nyl, case, seed):
    """Seeded initial fields written through view('i'): lock exchange (b = -0.5 | +0.5
    across x = L/2 plus uniform noise 1e-3) or Taylor-Green (u = sin x cos y cos z,
    v = -cos x sin y cos z plus Gaussian noise 1e-4, covariant: times the spacing)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = nyl.grid
    st = nyl.model.state
    if case == "lock":
        xb = g.x_b.view("i").numpy()
        b = np.where(xb < 0.5 * g.Lx, -0.5, 0.5) + 1e-3 * rng.uniform(-1, 1, size=xb.shape)
        st.b.view("i")[...] = torch.from_numpy(b)
    else:
        xu, yu, zu = (g.x_vel["i"].view("i").numpy(), g.y_vel["i"].view("i").numpy(), g.z_vel["i"].view("i").numpy())
        xv, yv, zv = (g.x_vel["j"].view("i").numpy(), g.y_vel["j"].view("i").numpy(), g.z_vel["j"].view("i").numpy())
        shape = xu.shape
        u = (np.sin(xu) * np.cos(yu) * np.cos(zu) + 1e-4 * rng.standard_normal(shape)) * g.dx
        v = (-np.cos(xv) * np.sin(yv) * np.cos(zv) + 1e-4 * rng.standard_normal(shape)) * g.dy
        w = 1e-4 * rng.standard_normal(shape) * g.dz
        st.u["i"].view("i")[...] = torch.from_numpy(u)
        st.u["j"].view("i")[...] = torch.from_numpy(v)
        st.u["k"].view("i")[...] = torch.from_numpy(w)


def footprint_bytes(case, n, precision="mixed"):
    """Device bytes of one run: 14 state fields, 3 x 4 time-scheme registers, and the
    multigrid workspace (x, b, y per level; in mixed precision also the float-pair
    solution and rhs of level 1 and the two float vectors of the Krylov solver), plus
    3% and 256 KiB for partial sums, scalars and allocator rounding."""
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
        mg += 2 * 8 * n ** 3 + 2 * 4 * n ** 3
    return int(1.03 * (fields + mg)) + (1 << 18)


def steps_per_graph(steps, kmax=10):
    """largest divisor of `steps` not above kmax: graph launches land exactly on `steps`"""
    for k in range(min(kmax, steps), 0, -1):
        if steps % k == 0:
            return k
    return 1


class Run:
    """One admitted request: resident state, its stream (of CUDA priority `priority`,
    lower = scheduled first) and its captured graph."""

    def __init__(self, req, precision, device, mg_tol, priority=0):
        self.req = req
        self.nyl = Nyles(build_params(req.case, req.n, precision, mg_tol), device=device)
        initial_state(self.nyl, req.case, req.seed)
        m = self.nyl.model
        m.diagnose_var(m.state)                       # core/nyles.py:122
        self.k = steps_per_graph(req.steps)
        m.capture_graph(CASES[req.case]["dt"], self.k)
        self.stream = torch.cuda.Stream(device=device, priority=priority)
        self.stream.wait_stream(torch.cuda.current_stream(device))
        self.launched = 0
        self.inflight = []                            # events of launches not yet seen complete
        self.last_event = None

    def launch(self):
        self.nyl.model.replay(stream=self.stream)
        ev = torch.cuda.Event()
        ev.record(self.stream)
        self.inflight.append(ev)
        self.last_event = ev
        self.launched += self.k

    def poll(self):
        while self.inflight and self.inflight[0].query():
            self.inflight.pop(0)
        return len(self.inflight)

    @property
    def all_launched(self):
        return self.launched >= self.req.steps

    def finished(self):
        return self.all_launched and self.poll() == 0

    def vcycles(self):
        return self.nyl.model.mg_stats()["vcycles"]

    def outcome(self):
        """(status, V-cycles) of a finished run: "blowup" when a pressure solve met a
        non-finite norm or the final velocity is not finite, "not_converged" when a
        solve stopped at maxite above the tolerance, else "ok"."""
        from . import _native as nat
        m = self.nyl.model
        s = m.mg_stats()
        status = "ok"
        if s["nonfinite"] > 0:
            status = "blowup"
        else:
            try:
                m.max_U2()
            except nat.BlowUp:
                status = "blowup"
        if status == "ok" and s["not_converged"] > 0:
            status = "not_converged"
        return status, s["vcycles"]

    def final_state(self):
        st = self.nyl.model.state
        return {s: st.get(s).view("i").double().cpu().numpy() for s in ("b", "u_i", "u_j", "u_k", "p")}


def remaining_work(run):
    """cells x steps not yet launched"""
    return run.req.n ** 3 * max(0, run.req.steps - run.launched)


class ServingEngine:
    """Admission against an HBM budget, resident runs, overlapping graph replays.

    priority "work" (default) gives each run's stream a CUDA priority by its total work
    (cells x steps): the GPU schedules the blocks of small runs first; "none" gives every
    stream the same priority. `window` = W advances only the W runs with the least
    remaining work at each tick (shortest remaining work first): small runs complete
    soon after they arrive, the large ones, which set the makespan, fill the device once
    the small ones are done; None advances every resident run."""

    def __init__(self, hbm_budget_bytes=120e9, precision="mixed", mg_tol=1e-6, device=None, inflight=2,
                 clock=time.perf_counter, run_factory=None, priority="work", window=None):
        if priority not in ("work", "none"):
            raise ValueError("priority must be 'work' or 'none'")
        if window is not None and window < 1:
            raise ValueError("window must be None or >= 1")
        self.priority = priority
        self.window = window
        self.budget = float(hbm_budget_bytes)
        self.precision = precision
        self.mg_tol = mg_tol
        self.run_factory = run_factory or Run
        if device is None and run_factory is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device) if device is not None else None
        self.inflight = inflight
        self.clock = clock
        self.used = 0
        self.peak_used = 0
        self.max_active = 0

    def serve(self, requests, realtime=True, keep_states=False):
        """Serve `requests` (arrival times relative to now when `realtime`, else all at
        once). Returns (results, final_states) with final_states[rid] = dict of numpy
        prognostic fields when keep_states."""
        pending = sorted(requests, key=lambda r: r.arrival)
        prio = self.stream_priorities(requests)
        queue, active, results, states = [], [], [], {}
        t0 = self.clock()
        nxt = 0
        while nxt < len(pending) or queue or active:
            now = self.clock() - t0
            while nxt < len(pending) and (not realtime or pending[nxt].arrival <= now):
                queue.append(pending[nxt])
                nxt += 1
            # admission: FIFO while the footprint fits; a request larger than the whole
            # budget is refused at once (it could never fit) and the queue moves on
            while queue:
                req = queue[0]
                need = footprint_bytes(req.case, req.n, self.precision)
                if need > self.budget:
                    queue.pop(0)
                    now = self.clock() - t0
                    results.append(Result(req.rid, req.case, req.n, req.steps, req.arrival if realtime else 0.0,
                                          now, now, req.n ** 3, 0, "refused"))
                    continue
                if self.used + need > self.budget and active:
                    break
                queue.pop(0)
                run = self.run_factory(req, self.precision, self.device, self.mg_tol, priority=prio[req.rid])
                run.admitted = self.clock() - t0
                run.need = need
                self.used += need
                self.peak_used = max(self.peak_used, self.used)
                active.append(run)
            self.max_active = max(self.max_active, len(active))
            # advance: keep up to `inflight` graph launches queued per run, for the
            # `window` runs with the least remaining work (all runs without a window)
            order = active if self.window is None else sorted(active, key=remaining_work)[:self.window]
            for run in order:
                if not run.all_launched and run.poll() < self.inflight:
                    run.launch()
            # completion
            still = []
            for run in active:
                if run.finished():
                    done = self.clock() - t0
                    req = run.req
                    status, vcycles = run.outcome()
                    results.append(Result(req.rid, req.case, req.n, req.steps, req.arrival if realtime else 0.0,
                                          run.admitted, done, req.n ** 3, vcycles, status))
                    if keep_states:
                        states[req.rid] = run.final_state()
                    self.used -= run.need
                    del run
                else:
                    still.append(run)
            active = still
            waiting = order if self.window is None else [r for r in order if r in active]
            if waiting and all(r.all_launched or r.poll() >= self.inflight for r in waiting):
                time.sleep(2e-4)
            elif not active and not queue and nxt < len(pending):
                time.sleep(max(0.0, min(2e-3, pending[nxt].arrival - (self.clock() - t0))))
        if self.device is not None and self.device.type == "cuda":
            torch.cuda.synchronize(self.device)
        return sorted(results, key=lambda r: r.rid), states

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
