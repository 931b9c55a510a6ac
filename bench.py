"""Benchmark of the Nyles time step on GB300: cell-steps/s at 256^3.

Workload (one GPU): Rayleigh-Taylor interface, 256x256x256 cells, box 1x1x1, periodic
in x and y, free-slip walls in z, b = +0.5 above z = 0.5 + eta(x, y) and -0.5 below
(eta: seeded Fourier modes 1 <= max(|kx|,|ky|) <= 8 scaled to max|eta| = 1e-2), fluid
at rest; RK3-SSP with dt = 1e-3; multigrid to sum(r^2)/sum(b^2) < 1e-20 (relative
residual 1e-10). A step = one full RK3 step (3 right-hand sides, 3 projections).
`value` is the FP64 path with the state resident on the device; `mixed` reports the
mixed-precision path (FP32 state and stencils, FP32 V-cycles in FP64 refinement) on
the same workload, and its error against the FP64 path after 100 steps from the same
state (`mixed.accuracy`). `e2e` runs the same steps through the public API with the
prognostic state copied in from pinned host memory and copied back every step.
`step_roofline` = algorithmic bytes per cell-step (RK3 stencil part plus three
multigrid solves at the measured V-cycle count) x cell-steps/s against the measured HBM
copy bandwidth; `roofline` = the dominant kernel alone.

`serving`: an ensemble of 96 lock-exchange and Taylor-Green runs on n^3 grids,
n in {32, 48, 64, 96, 128}, arriving as a seeded Poisson stream at 20 per second,
mixed precision, served by continuous batching under a 120 GB HBM budget; p50/p99
completion latency and aggregate cell-steps/s, against the same runs one at a time
with the eager FP64 path (each run's duration from the measured setup and step times
of its case and grid). Each run lasts --serving-steps steps (300 by default).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--n 256]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

# more hardware work queues for the serving ensemble's many streams (read when the CUDA
# context is created; the timed single-stream steps do not depend on it)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cell-steps/s at 256^3 (FP64 vs mixed, same error); ensemble p50/p99 latency"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="cells per direction")
    ap.add_argument("--precision", default="both", choices=["fp64", "mixed", "both"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=2, help="extra steps timed per phase with CUDA events")
    ap.add_argument("--serving-requests", type=int, default=96, help="0 skips the serving ensemble")
    ap.add_argument("--serving-steps", type=int, default=300, help="time steps of each ensemble run")
    ap.add_argument("--serving-rate", type=float, default=20.0, help="Poisson arrivals per second")
    ap.add_argument("--no-serving-baseline", action="store_true")
    ap.add_argument("--serving-priority", default="work", choices=["work", "none"],
                    help="CUDA stream priority of each run by its total work, or none")
    ap.add_argument("--serving-capacity", default="auto",
                    help="slots per size bucket (runs advanced by one batched launch): 1..32, or auto (as many "
                         "n^3 runs as 2^23 cells hold)")
    ap.add_argument("--serving-sequential", default="estimate", choices=["estimate", "measured"],
                    help="sequential FP64 baseline: bucket timings replayed over the queue, or every run executed")
    ap.add_argument("--no-eager", action="store_true", help="skip the eager (no graph) timing beside the headline")
    ap.add_argument("--accuracy-steps", type=int, default=100,
                    help="steps of the mixed-vs-FP64 error check (0 skips it)")
    ap.add_argument("--configs", action="store_true",
                    help="instead of the headline: FP64 and mixed throughput, V-cycles and mixed-vs-FP64 error of "
                         "each workload configuration (lock exchange, Taylor-Green, Rayleigh-Taylor, shear)")
    return ap.parse_args()


# ------------------------------------------------------------------ workload
def rt_params(n, precision):
    from nyles_gb300 import parameters
    parameters.InextensibleDict.unfreeze()
    p = parameters.UserParameters()
    p.model["modelname"] = "LES"
    p.model["geometry"] = "perio_xy"
    p.model["Lx"], p.model["Ly"], p.model["Lz"] = 1.0, 1.0, 1.0
    p.time["timestepping"] = "RK3_SSP"
    p.time["auto_dt"] = False
    p.time["dt"] = 1e-3
    p.discretization["global_nx"] = n
    p.discretization["global_ny"] = n
    p.discretization["global_nz"] = n
    p.gpu["precision"] = precision
    p.gpu["mg_tol"] = 1e-20
    p.gpu["mg_maxite"] = 40
    p.gpu["history"] = False
    return p


def rt_interface(grid, seed=3, kmax=8, amp=1e-2):
    """eta(x, y) on the cell centres of the array (z, y, x) broadcast."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    x = grid.x_b_1D / grid.Lx
    y = grid.y_b_1D / grid.Ly
    X, Y = np.meshgrid(x, y, indexing="xy")
    eta = np.zeros_like(X)
    for kx in range(-kmax, kmax + 1):
        for ky in range(-kmax, kmax + 1):
            if 1 <= max(abs(kx), abs(ky)) <= kmax:
                a, b = rng.standard_normal(2)
                ph = 2 * np.pi * (kx * X + ky * Y)
                eta += a * np.cos(ph) + b * np.sin(ph)
    return eta * (amp / np.abs(eta).max())


def rt_init(nyl):
    import numpy as np
    import torch
    g = nyl.grid
    eta = rt_interface(g)
    zb = g.z_b_1D[:, None, None]
    b = np.where(zb > 0.5 * g.Lz + eta[None, :, :], 0.5, -0.5)
    nyl.model.state.b.view("i")[...] = torch.from_numpy(b)


def build_model(n, precision):
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(rt_params(n, precision))
    rt_init(nyl)
    return nyl


# ------------------------------------------------------------------ measurement helpers
class ClockSampler:
    """nvidia-smi samples (200 ms) while running; median SM clock and active reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import statistics
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops():
    """Measured double-precision rate of this GPU: cuBLAS DGEMM (torch.mm float64),
    best of 5, 2*n^3 flops. GB300's FP64 rate is a small fraction of its FP32 rate,
    which bounds every FP64 stencil here before HBM bandwidth does."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def mg_levels(n):
    """Interior extents of the multigrid levels of an n^3 perio_xy grid (x, y halve
    until 2; z interior halves alongside)."""
    levels, x, z = [], n, n
    while True:
        levels.append((z, x, x))
        if x == 2:
            break
        x //= 2
        z //= 2
    return levels


# FP64 flops (DADD + DMUL + 2 x DFMA thread instructions) per interior cell of one
# k_rhs_march<double, 1, 1, 0> launch, counted by ncu on the 128^3 case of this workload
# (smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on: 223.5 + 237.8 + 2 x 237.5
# per cell), and the FP64 instructions (issue slots) behind them
RHS_FP64_OPS_PER_CELL = 936
RHS_FP64_INSTR_PER_CELL = 699
# DRAM bytes (read + write) per interior cell of one launch: ncu, FP64 at 128^3
# (159.0 + 43.7 MB), mixed (k_rhs_les) at 256^3 (614.8 + 257.5 MB)
RHS_DRAM_BYTES_PER_CELL = {8: 202.72e6 / 128 ** 3, 4: 872.35e6 / 256 ** 3}
# DRAM bytes of one level-0 Jacobi half-sweep launch at 256^3, mixed (ncu, vector form:
# 134.3 + 40.9 MB; algorithmic 201.3 MB, the rest of the output still in L2 at the end)
JACOBI_F32_L0_DRAM_BYTES_256 = 175.2e6


def mg_bottom_level(levels, elem, smem=200 * 1024, maxvol_fp64=1024):
    """First level of the one-block coarse solve (the library's rule: the coarsest
    levels whose x, b, y fit in `smem` bytes, two levels at least, never level 0; in
    FP64 no level above `maxvol_fp64` cells)."""
    L = len(levels)
    bottom, total = L, 0
    for l in range(L - 1, 0, -1):
        z, y, x = levels[l]
        total += 3 * z * y * x * elem
        if total > smem:
            break
        if elem == 8 and z * y * x > maxvol_fp64:
            break
        if L - l >= 2:
            bottom = l
    return bottom


def roofline(kernel, ph, n, elem, peak, peak_kind, fp64_peak, nv=None, solves=None, krylov=False):
    """Roofline of one kernel family from the CUDA-event phase times.

    rhs       : one launch reads b, U(3), vor(3), ke and writes 4 registers: 12 words
                per interior cell (the periodic halo's tendencies are not computed). In FP64 the kernel is bound by the FP64
                pipe (GB300 issues FP64 at 1/64 of its FP32 rate): the roofline is
                then the FP64 arithmetic rate against cuBLAS DGEMM, with the
                issue-slot fraction (DADD and DMUL take a slot for one flop, DFMA for
                two) and the HBM figures beside it.
    mg_smooth : each Jacobi half-sweep reads its input and b and writes its output, 3
                words per level cell; per V-cycle, on each grid level above the
                one-block coarse levels: 3 half-sweeps (the first of the pre-smoothing
                is written by the kernel that sets b; FP64 level 0, warm-started: 4),
                plus, in mixed precision, the float-pair solution read and written by
                the last level-0 half-sweep (16 B per cell; the Krylov solve instead
                reads q, 4 B); the one-block coarse solve reads b and writes x of its
                first level.
    mg_norm   : mixed precision, the float-pair outer iteration per solve and level-0
                cell: sum(b^2) 8 B, nv + 1 residuals of 24 B, and per Krylov iteration
                the direction update (24 B) and the solution update (20 B).
    """
    if ph.get(kernel, {}).get("count", 0) == 0:
        return None
    ms = ph[kernel]["ms"]
    out = {"kernel": kernel, "bound": "hbm", "peak": peak, "unit": "GB/s", "peak_kind": peak_kind, "traffic": None}
    if kernel == "rhs":
        vol = n ** 3   # the time step computes the b and u tendencies of interior cells only
        launches = ph[kernel]["count"]
        per_launch = 12 * elem * vol
        avg = ms / launches
        hbm = {"achieved": per_launch / (avg * 1e-3) / 1e9, "peak": peak, "unit": "GB/s", "peak_kind": peak_kind,
               "bytes_per_launch": per_launch, "traffic": RHS_DRAM_BYTES_PER_CELL[elem] * vol,
               "traffic_source": "ncu dram bytes per cell of the same kernel, scaled to this grid"}
        hbm["frac"] = hbm["achieved"] / peak
        if elem == 8 and fp64_peak:
            flops = RHS_FP64_OPS_PER_CELL * vol / (avg * 1e-3) / 1e12
            issue = RHS_FP64_INSTR_PER_CELL * vol / (avg * 1e-3) / 1e12
            return {"kernel": "k_rhs_march", "bound": "fp64", "achieved": flops, "peak": fp64_peak,
                    "unit": "TFLOP/s", "peak_kind": "measured (cuBLAS DGEMM, torch.mm float64 8192^3)",
                    "frac": flops / fp64_peak, "fp64_flops_per_cell": RHS_FP64_OPS_PER_CELL,
                    "fp64_instructions_per_cell": RHS_FP64_INSTR_PER_CELL,
                    "fp64_issue_frac": issue / (fp64_peak / 2), "avg_launch_ms": avg,
                    "traffic": hbm["traffic"], "hbm": hbm}
        out.update({"kernel": "k_rhs_march", "avg_launch_ms": avg})
        out.update({k: v for k, v in hbm.items() if k not in ("peak", "unit", "peak_kind", "frac")})
    elif kernel == "mg_smooth":
        lev = mg_levels(n)
        B = mg_bottom_level(lev, elem)
        vol = [z * y * x for (z, y, x) in lev]
        per_vcycle = sum((4 if (l == 0 and elem == 8) else 3) * 3 * elem * vol[l] for l in range(B))
        if elem == 4:
            per_vcycle += (4 if krylov else 16) * vol[0]
        if B < len(lev):
            per_vcycle += 2 * elem * vol[B]
        calls_per_vcycle = 2 * B + 1   # one bracketed call per smoothing and the coarse solve
        vcycles = ph[kernel]["count"] / calls_per_vcycle
        total = per_vcycle * vcycles
        out.update({"kernel": "k_mg_jacobi (+ k_mg_bottom)", "bytes_per_vcycle": per_vcycle, "vcycles": vcycles,
                    "ms_per_vcycle": ms / vcycles, "achieved": total / (ms * 1e-3) / 1e9})
        if elem == 4 and n == 256:
            out["traffic"] = JACOBI_F32_L0_DRAM_BYTES_256
            out["traffic_source"] = ("ncu dram bytes of one level-0 half-sweep launch (algorithmic %.1f MB)"
                                     % (3 * 4 * vol[0] / 1e6))
    elif kernel == "mg_norm" and elem == 4 and nv is not None and solves:
        v0 = n ** 3
        per_solve = v0 * (8 + (nv + 1) * 24 + (nv * 44 if krylov else 0))
        out.update({"kernel": "k_mg_resid_df" + (" + k_fcg_direction + k_fcg_xupdate" if krylov else ""),
                    "bytes_per_solve": per_solve, "solves": solves,
                    "achieved": per_solve * solves / (ms * 1e-3) / 1e9})
    else:
        out["achieved"] = None
    if out.get("achieved") is not None:
        out["frac"] = out["achieved"] / peak
    return out


# ------------------------------------------------------------------ timed runs
def time_steps(nyl, K, W, stream, graphs=True):
    """K timed steps of model.forward after W warm-up steps; with graphs, forward
    replays its captured fixed-dt step (the path Nyles.run takes), without them every
    step is launched eagerly with the multigrid stop test on the host."""
    import torch
    m = nyl.model
    m.use_graphs = graphs
    for _ in range(W):
        m.forward(0.0, nyl.dt0)
    torch.cuda.synchronize()
    st0 = m.mg_stats()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    from nyles_gb300 import _native
    l0 = _native.lib().nyles_launch_count()
    start.record(stream)
    for _ in range(K):
        m.forward(0.0, nyl.dt0)
    end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    st1 = m.mg_stats()
    launches = _native.lib().nyles_launch_count() - l0
    vc = (st1["vcycles"] - st0["vcycles"]) / max(1, (st1["solves"] - st0["solves"]))
    return ms, launches, vc


def profile_phases(nyl, steps):
    import ctypes
    import torch
    from nyles_gb300 import _native as nat
    m = nyl.model
    lib = nat.lib()
    m.profile(True)
    for _ in range(steps):
        m.forward(0.0, nyl.dt0)
    torch.cuda.synchronize()
    ms = (ctypes.c_double * nat.NPHASE)()
    cnt = (ctypes.c_longlong * nat.NPHASE)()
    nat.check(lib.nyles_model_profile_read(m._h, ms, cnt, nat.NPHASE))
    m.profile(False)
    return {nat.PHASES[i]: {"ms": ms[i], "count": cnt[i]} for i in range(nat.NPHASE)}


def time_e2e(nyl, K, W):
    """Same steps through the public API, prognostic state in pinned host memory."""
    import torch
    m = nyl.model
    names = m.state.get_prognostic_scalars()
    dev = [m.state.get(s).data for s in names]
    host = [torch.empty_like(t, device="cpu").pin_memory() for t in dev]
    for h, d in zip(host, dev):
        h.copy_(d)
    bytes_in = sum(h.numel() * h.element_size() for h in host)

    def step():
        for h, d in zip(host, dev):
            d.copy_(h, non_blocking=True)
        m.forward(0.0, nyl.dt0)
        for h, d in zip(host, dev):
            h.copy_(d, non_blocking=True)

    for _ in range(W):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        step()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) * 1e3, bytes_in


def time_serving(a):
    """Serving ensemble: seeded Poisson stream of lock-exchange and Taylor-Green runs on
    n^3 grids, n in {32, 48, 64, 96, 128}, mixed precision, admitted against a 120 GB
    budget into size buckets advanced by batched graph launches; baseline = the same runs
    one at a time with the FP64 path (model.forward): with "estimate" the setup and step
    time of each (case, grid) are measured and the arrival queue is replayed with them,
    with "measured" every run is executed (about four minutes for the 96 runs)."""
    import torch
    from nyles_gb300 import serving as S
    warm = [S.Request(i, c, n, i, 4, 0.0) for i, (c, n) in enumerate((("lock", 32), ("tgv", 32)))]
    S.ServingEngine(precision="mixed").serve(warm, realtime=False)
    reqs = S.make_requests(a.serving_requests, a.serving_rate, seed=5, steps=a.serving_steps)
    cap = a.serving_capacity if a.serving_capacity == "auto" else int(a.serving_capacity)
    eng = S.ServingEngine(hbm_budget_bytes=120e9, precision="mixed", priority=a.serving_priority, capacity=cap)
    from nyles_gb300 import _native
    l0 = _native.lib().nyles_launch_count()
    torch.cuda.synchronize()
    res, _ = eng.serve(reqs, realtime=True)
    launches = _native.lib().nyles_launch_count() - l0
    out = {"requests": len(reqs), "steps_per_run": a.serving_steps, "rate_per_s": a.serving_rate,
           "stream_seed": 5, "sizes": [32, 48, 64, 96, 128], "precision": "mixed", "mg_tol_sq_ratio": 1e-6,
           "hbm_budget_gb": 120, "stream_priority": a.serving_priority,
           "bucket_capacity": ({str(n): S.auto_capacity(n) for n in (32, 48, 64, 96, 128)} if cap == "auto" else cap),
           "buckets": eng.buckets_made, "batched_launches": eng.launches,
           "max_resident_runs": eng.max_active, "peak_footprint_gb": eng.peak_used / 1e9,
           "kernel_launches": launches}
    out.update(S.summarize(res))
    if not a.no_serving_baseline and a.serving_sequential == "measured":
        seq, _ = S.run_sequential(reqs, precision="fp64")
        out["sequential_fp64"] = S.summarize(seq)
        out["sequential_fp64"]["method"] = ("every run executed one at a time in arrival order with the FP64 path "
                                            "(model.forward: graph replay after its second step); a run starts at "
                                            "max(arrival, end of the previous run)")
    elif not a.no_serving_baseline:
        seq, timing = S.sequential_estimate(reqs, precision="fp64")
        out["sequential_fp64"] = S.summarize(seq)
        out["sequential_fp64"]["method"] = ("setup and FP64 step time measured per (case, grid) bucket "
                                            "(10 steps after 2), arrival queue replayed one run at a time")
        out["sequential_fp64"]["step_ms"] = {"%s_%d" % k: round(v["step_s"] * 1e3, 3) for k, v in timing.items()}
    torch.cuda.empty_cache()
    return out


def oracle_rt(n, threads=1):
    """The CPU oracle (C++ restatement of the reference's numerics, its loops on
    `threads` host threads; 0 = all) set up with the Rayleigh-Taylor workload at n^3 and
    projected once."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(threads)
    import numpy as np
    from nyles_gb300 import grid as grid_module
    from nyles_gb300 import topology as topo
    prm = dict(nx=n, ny=n, nz=n, nh=3, npx=1, npy=1, npz=1, Lx=1.0, Ly=1.0, Lz=1.0, loc=[0, 0, 0],
               neighbours=topo.get_neighbours([0, 0, 0], [1, 1, 1], "perio_xy"))
    g = grid_module.Grid(prm)
    o = oracle.OracleModel(dict(nx=n, ny=n, nz=n, geometry="perio_xy", timestepping="RK3_SSP", dx=g.dx, dy=g.dy,
                                dz=g.dz, idx2=g.idx2, idy2=g.idy2, idz2=g.idz2))
    o.mg_params(1e-20, 40, 0.9)
    eta = rt_interface(g)
    zb = g.z_b_1D[:, None, None]
    o.field("b")[...] = np.where(zb > 0.5 + eta[None, :, :], 0.5, -0.5)
    o.diagnose()
    return o


def cpu_baseline(nsample=256, steps=1):
    """The oracle on one host core (the reference runs one thread per subdomain):
    `steps` RK3 steps of the workload at nsample^3 after its initial projection."""
    o = oracle_rt(nsample, threads=1)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.forward(0.0, 1e-3)
    el = time.perf_counter() - t0
    return {"value": nsample ** 3 * steps / el, "unit": "cell-steps/s", "cores": 1, "kind": "port",
            "sample": "oracle (C++ restatement of the reference numerics, 1 thread) on the same Rayleigh-Taylor "
                      "setup at %d^3, %d RK3 step(s), %.1f s" % (nsample, steps, el)}


# ------------------------------------------------------------------ reference arm
REFERENCE_BUDGET_S = 150.0   # bound of the timed steps of the reference arm


def run_reference(a, rank, world):
    """The reference's numerics on the host cores, on this arm's workload (the same
    grid, setup and solver tolerance): the oracle, its stencil and multigrid sweeps split
    over every host thread (the reference would run one MPI rank per core on as many
    subdomains; one subdomain on all cores is the same machine's CPU throughput for this
    grid). One untimed step, then up to K timed RK3 steps, stopped early once
    REFERENCE_BUDGET_S seconds have passed (each step of the 256^3 grid takes seconds);
    value = cells x timed steps / their time."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = a.n
    o = oracle_rt(n, threads=0)
    for _ in range(min(a.warmup, 1)):
        o.forward(0.0, 1e-3)
    t0 = time.perf_counter()
    done = 0
    while done < a.steps:
        o.forward(0.0, 1e-3)
        done += 1
        if time.perf_counter() - t0 > REFERENCE_BUDGET_S:
            break
    el = time.perf_counter() - t0
    value = float(n ** 3 * done / el)
    sample = ("the oracle (C++ restatement of the reference numerics; the reference's Fortran path cannot be built "
              "here) on this arm's Rayleigh-Taylor workload at %d^3, loops on %d host threads, %d timed RK3 step(s) "
              "of the %d requested after %d untimed, %.1f s" % (n, threads, done, a.steps, min(a.warmup, 1), el))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": a.gpus,
            "steps": a.steps, "timed_steps": done, "warmup": a.warmup, "ms_per_step": el * 1e3 / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": make_config(n, world),
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def job_time_ms(ms, dist=None, device="cpu"):
    """Time of the whole job: the maximum over ranks of each rank's timed region."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(cells, steps, ms, world):
    """Whole-job cell-steps/s: every replica advances `cells` cells by `steps` steps."""
    return world * cells * steps / (ms * 1e-3)


def make_config(n, world):
    return {"workload": "rayleigh_taylor_%d^3_perio_xy_rk3" % n, "grid": [n, n, n], "box": [1, 1, 1],
            "dt": 1e-3, "mg_tol_sq_ratio": 1e-20, "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (state >> 129 MB)"}


def accuracy(n, steps):
    """Mixed path against the FP64 path after `steps` RK3 steps from the same state:
    max|mixed - fp64| / max|fp64| for b and p, and over the three components for u.
    The pressure of a box closed or periodic on every side is defined up to a constant,
    which the Krylov solve and the stationary V-cycle iteration fix differently (the
    velocity correction uses its gradient only): p is compared after removing each
    field's mean."""
    import numpy as np
    import torch
    fields = ("b", "p", "u_i", "u_j", "u_k")
    out = {}
    for prec in ("fp64", "mixed"):
        nyl = build_model(n, prec)
        m = nyl.model
        m.diagnose_var(m.state)
        for _ in range(steps):
            m.forward(0.0, nyl.dt0)
        torch.cuda.synchronize()
        out[prec] = {s: m.state.get(s).view("i").double().cpu().numpy() for s in fields}
        del nyl, m
        torch.cuda.empty_cache()
    a, b = out["mixed"], out["fp64"]
    for d in (a, b):
        d["p"] = d["p"] - d["p"].mean()
    err = {s: float(np.abs(a[s] - b[s]).max() / max(np.abs(b[s]).max(), 1e-300)) for s in ("b", "p")}
    us = max(np.abs(b[c]).max() for c in ("u_i", "u_j", "u_k"))
    err["u"] = float(max(np.abs(a[c] - b[c]).max() for c in ("u_i", "u_j", "u_k")) / max(us, 1e-300))
    return {"steps": steps, "rel_err_vs_fp64": err}


def step_bytes(prec, nv, n_vcycles, refine=True, krylov=False):
    """Algorithmic bytes per cell-step: RK3 stencil part w(11 nv + 6) plus 3 solves of
    w_mg (4 + 24 n_V), and, in mixed precision, per cell and V-cycle of the float-pair
    outer iteration: 40 B for iterative refinement (residual 24, correction 16), 72 B
    for the Krylov solve (residual 24, z.q read 4, direction and image update 24,
    solution update 20)."""
    w = 8 if prec == "fp64" else 4
    q = w * (11 * nv + 6) + 3 * w * (4 + 24 * n_vcycles)
    if prec != "fp64" and refine:
        q += 3 * (72 if krylov else 40) * n_vcycles
    return q


# ------------------------------------------------------------------ configuration table
TWO_PI = 6.283185307179586


def config_params(name, precision):
    """Parameters of a workload configuration: lock exchange 64x32x32 in 4x1x1 (closed,
    RK3, dt 2e-3, reference tolerances), Taylor-Green 128^3 (triply periodic box 2 pi, RK3,
    dt 5e-3, relative residual 1e-10), Rayleigh-Taylor 256x256x512 (box 1x1x2, perio_xy,
    dt 1e-3, relative residual 1e-10), stratified shear 512x256x256 with a tracer (box
    4x2x1, perio_xy, adaptive CFL 0.8)."""
    from nyles_gb300 import parameters
    parameters.InextensibleDict.unfreeze()
    p = parameters.UserParameters()
    c = {"lock": dict(geometry="closed", n=(64, 32, 32), L=(4.0, 1.0, 1.0), dt=2e-3, tol=1e-6, maxite=20),
         "tgv": dict(geometry="perio_xyz", n=(128, 128, 128), L=(TWO_PI,) * 3, dt=5e-3, tol=1e-20, maxite=40),
         "rt": dict(geometry="perio_xy", n=(256, 256, 512), L=(1.0, 1.0, 2.0), dt=1e-3, tol=1e-20, maxite=40),
         "shear": dict(geometry="perio_xy", n=(512, 256, 256), L=(4.0, 2.0, 1.0), dt=None, tol=1e-6, maxite=20,
                       ntr=1)}[name]
    p.model["modelname"] = "LES"
    p.model["geometry"] = c["geometry"]
    p.model["Lx"], p.model["Ly"], p.model["Lz"] = c["L"]
    p.model["n_tracers"] = c.get("ntr", 0)
    p.time["timestepping"] = "RK3_SSP"
    p.time["auto_dt"] = c["dt"] is None
    p.time["dt"] = c["dt"] or 1.0
    p.time["cfl"] = 0.8
    p.time["dt_max"] = 1.0
    p.discretization["global_nx"], p.discretization["global_ny"], p.discretization["global_nz"] = c["n"]
    p.gpu["precision"] = precision
    p.gpu["mg_tol"] = c["tol"]
    p.gpu["mg_maxite"] = c["maxite"]
    p.gpu["history"] = False
    return p


def config_init(name, nyl):
    """Seeded initial state of a configuration (covariant velocities, walls at rest)."""
    import numpy as np
    import torch
    from nyles_gb300 import serving
    if name == "lock":
        serving.initial_state(nyl, "lock", 1)
    elif name == "tgv":
        serving.initial_state(nyl, "tgv", 2)
    elif name == "rt":
        rt_init(nyl)
    else:
        g = nyl.grid
        st = nyl.model.state
        rng = np.random.Generator(np.random.PCG64(4))
        zb = g.z_b.view("i").numpy()
        zu = g.z_vel["i"].view("i").numpy()
        U0 = 0.05 * np.sqrt(5.0)    # minimum Richardson number 0.2 at N^2 = 1
        st.get("u_i").view("i")[...] = torch.from_numpy(U0 * np.tanh((zu - 0.5) / 0.05) * g.dx)
        st.get("b").view("i")[...] = torch.from_numpy(zb.copy())
        st.get("t0").view("i")[...] = torch.from_numpy(np.tanh((zb - 0.5) / 0.05))
        v = 1e-3 * rng.standard_normal(zb.shape) * g.dy
        w = 1e-3 * rng.standard_normal(zb.shape) * g.dz
        w[-1, :, :] = 0.0
        st.get("u_j").view("i")[...] = torch.from_numpy(v)
        st.get("u_k").view("i")[...] = torch.from_numpy(w)


def run_config(name, precision, steps, warmup, err_steps):
    """Timed steps of one configuration (graph replay; adaptive dt: eager steps with the
    CFL reduction, as Nyles.run takes them), then err_steps steps from the initial state
    whose final fields are returned for the mixed-vs-FP64 comparison. Stops at a blow-up
    (NYLES_BLOWUP or a non-finite CFL reduction) and reports its step."""
    import numpy as np
    import torch
    from nyles_gb300 import _native as nat
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(config_params(name, precision))
    config_init(name, nyl)
    m = nyl.model
    m.diagnose_var(m.state)
    cells = nyl.param["nx"] * nyl.param["ny"] * nyl.param["nz"]
    out = {"cells": cells}

    def step(t):
        try:
            dt = nyl.compute_dt()
        except nat.BlowUp:
            return None
        return dt if not m.forward(t, dt) else None

    # error trajectory from the initial state (the timed steps of a fixed-dt case come
    # after it; an adaptive-dt case is timed on it, after `warmup` steps, up to a blow-up)
    t, blow = 0.0, None
    s0 = m.mg_stats()
    traj_ms, traj_steps = 0.0, 0
    for k in range(err_steps):
        if nyl.auto_dt:
            torch.cuda.synchronize()
            tk = time.perf_counter()
        dt = step(t)
        if dt is None:
            blow = k + 1
            break
        if nyl.auto_dt and k >= warmup:
            torch.cuda.synchronize()
            traj_ms += (time.perf_counter() - tk) * 1e3
            traj_steps += 1
        t += dt
    torch.cuda.synchronize()
    if nyl.auto_dt and traj_steps:
        out["path"] = "eager steps, adaptive dt (CFL reduction read back every step)"
        out["timed_steps"] = traj_steps
        out["ms_per_step"] = traj_ms / traj_steps
        out["cell_steps_per_s"] = cells * traj_steps / (traj_ms * 1e-3)
    s1 = m.mg_stats()
    out["mean_vcycles_per_solve"] = (s1["vcycles"] - s0["vcycles"]) / max(1, s1["solves"] - s0["solves"])
    names = ["b", "u_i", "u_j", "u_k", "p"] + ["t%d" % i for i in range(nyl.param["n_tracers"])]
    fields = {s: m.state.get(s).view("i").double().cpu().numpy() for s in names}
    out["err_steps"] = err_steps if blow is None else blow
    if blow is not None or nyl.auto_dt:
        if blow is not None:
            out["blowup_step"] = blow
        del nyl, m
        torch.cuda.empty_cache()
        return out, fields
    if name != "shear":
        fields_ok = all(np.isfinite(v).all() for v in fields.values())
        out["finite"] = bool(fields_ok)
    # timed steps (continuing the trajectory)
    stream = torch.cuda.current_stream()
    if nyl.auto_dt:
        for _ in range(warmup):
            t += step(t) or 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        done = 0
        for _ in range(steps):
            dt = step(t)
            if dt is None:
                break
            t += dt
            done += 1
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3
        out["path"] = "eager steps, adaptive dt (CFL reduction read back every step)"
    else:
        ms, _, _ = time_steps(nyl, steps, warmup, stream)
        done = steps
        out["path"] = "graph replay"
    out["timed_steps"] = done
    if done:
        out["ms_per_step"] = ms / done
        out["cell_steps_per_s"] = cells * done / (ms * 1e-3)
    del nyl, m
    torch.cuda.empty_cache()
    return out, fields


def config_table(a):
    """FP64 and mixed throughput of each configuration and the mixed path's relative
    max-norm error in b, u (velocity vector) and p (means removed) against the FP64
    path after the same number of steps from the same state."""
    import numpy as np
    plan = {"lock": (4, 1, 5), "tgv": (20, 3, 200), "rt": (10, 3, 100), "shear": (10, 1, 8)}
    table = {}
    for name, (steps, warmup, err_steps) in plan.items():
        row = {}
        runs = {}
        for prec in ("fp64", "mixed"):
            row[prec], runs[prec] = run_config(name, prec, steps, warmup, err_steps)
        f, g = runs["mixed"], runs["fp64"]
        if ("blowup_step" not in row["fp64"] and "blowup_step" not in row["mixed"]
                and all(np.isfinite(v).all() for v in list(f.values()) + list(g.values()))):
            err = {}
            for s in ("b", "p") + tuple(k for k in f if k.startswith("t")):
                x, y = f[s], g[s]
                if s == "p":
                    x, y = x - x.mean(), y - y.mean()
                err[s] = float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))
            us = max(np.abs(g[c]).max() for c in ("u_i", "u_j", "u_k"))
            err["u"] = float(max(np.abs(f[c] - g[c]).max() for c in ("u_i", "u_j", "u_k")) / max(us, 1e-300))
            row["mixed_vs_fp64"] = {"steps": min(row["fp64"]["err_steps"], row["mixed"]["err_steps"]),
                                    "rel_err": err}
        if "cell_steps_per_s" in row["fp64"] and "cell_steps_per_s" in row["mixed"]:
            row["mixed_speedup"] = row["mixed"]["cell_steps_per_s"] / row["fp64"]["cell_steps_per_s"]
        table[name] = row
        print(json.dumps({name: row}), flush=True)
    return table


# ------------------------------------------------------------------ main
def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    if a.configs:
        print(json.dumps({"configs": config_table(a)}))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    n = a.n
    cells = n ** 3
    peak, peak_kind = peaks()
    fp64_peak = fp64_peak_tflops() if a.precision in ("fp64", "both") else None
    out = {"metric": METRIC, "unit": "cell-steps/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic",
           "config": make_config(n, world)}
    results = {}
    precs = ["fp64", "mixed"] if a.precision == "both" else [a.precision]
    launches_total = 0
    with ClockSampler(local) as clk:
        for prec in precs:
            nyl = build_model(n, prec)
            nyl.model.diagnose_var(nyl.model.state)
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            ms, launches, vc = time_steps(nyl, a.steps, a.warmup, stream)
            ms = job_time_ms(ms, dist, "cuda")
            launches_total += launches
            res = {"ms_per_step": ms / a.steps, "value": job_value(cells, a.steps, ms, world),
                   "mean_vcycles_per_solve": vc, "kernel_launches": launches, "path": "graph replay",
                   "krylov": bool(getattr(nyl.model, "krylov", False))}
            if not a.no_eager:
                ems_eager, _, _ = time_steps(nyl, a.steps, 1, stream, graphs=False)
                ems_eager = job_time_ms(ems_eager, dist, "cuda")
                res["eager"] = {"ms_per_step": ems_eager / a.steps,
                                "value": job_value(cells, a.steps, ems_eager, world),
                                "note": "same steps launched one kernel at a time, multigrid stop test on the host"}
            if a.profile_steps > 0:
                res["phases"] = profile_phases(nyl, a.profile_steps)
            nyl.model.use_graphs = True
            if not a.no_e2e:
                ems, bts = time_e2e(nyl, max(1, a.steps // 2), 1)
                k = max(1, a.steps // 2)
                res["e2e"] = {"value": world * cells * k / (ems * 1e-3), "unit": "cell-steps/s",
                              "h2d_bytes_per_step": bts, "d2h_bytes_per_step": bts}
            results[prec] = res
            del nyl
            torch.cuda.empty_cache()
    clocks = clk.summary()
    main_prec = "fp64" if "fp64" in results else precs[0]
    r = results[main_prec]
    out.update({"value": r["value"], "ms_per_step": r["ms_per_step"],
                "dtype": "f64" if main_prec == "fp64" else "f32+f64", "clocks": clocks,
                "gpu_launches": launches_total, "mg": {"mean_vcycles_per_solve": r["mean_vcycles_per_solve"]},
                "path": r["path"], "eager": r.get("eager")})
    if "e2e" in r:
        out["e2e"] = r["e2e"]
    # roofline of the dominant kernel (largest share of device time)
    if "phases" in r:
        ph = r["phases"]
        kernels = {k: v for k, v in ph.items() if k not in ("mg_solve",)}
        dom = max(kernels, key=lambda k: kernels[k]["ms"])
        elem = 8 if main_prec == "fp64" else 4
        out["phases"] = {k: round(v["ms"] / max(1, a.profile_steps), 3) for k, v in ph.items()}
        kw = dict(nv=r["mean_vcycles_per_solve"], solves=3 * a.profile_steps, krylov=r.get("krylov", False))
        out["roofline"] = roofline(dom, ph, n, elem, peak, peak_kind, fp64_peak, **kw)
        out["roofline_kernels"] = {k: roofline(k, ph, n, elem, peak, peak_kind, fp64_peak, **kw)
                                   for k in ("rhs", "mg_smooth", "mg_norm") if k != dom}
    if "mixed" in results and main_prec != "mixed":
        mr = results["mixed"]
        out["mixed"] = {"value": mr["value"], "ms_per_step": mr["ms_per_step"],
                        "speedup_vs_fp64": mr["value"] / r["value"],
                        "mean_vcycles_per_solve": mr["mean_vcycles_per_solve"], "eager": mr.get("eager"),
                        "solver": ("FCG(1) preconditioned by the FP32 V-cycle" if mr["krylov"]
                                   else "stationary V-cycle iteration (iterative refinement)")}
        if "e2e" in mr:
            out["mixed"]["e2e"] = mr["e2e"]
        if "phases" in mr:
            mph = mr["phases"]
            out["mixed"]["phases"] = {k: round(v["ms"] / max(1, a.profile_steps), 3) for k, v in mph.items()}
            mdom = max((k for k in mph if k != "mg_solve"), key=lambda k: mph[k]["ms"])
            kw = dict(nv=mr["mean_vcycles_per_solve"], solves=3 * a.profile_steps, krylov=mr.get("krylov", False))
            out["mixed"]["roofline"] = roofline(mdom, mph, n, 4, peak, peak_kind, None, **kw)
            out["mixed"]["roofline_kernels"] = {k: roofline(k, mph, n, 4, peak, peak_kind, None, **kw)
                                                for k in ("rhs", "mg_smooth", "mg_norm") if k != mdom}
    if a.serving_requests > 0:
        out["serving"] = time_serving(a)
        out["gpu_launches"] += out["serving"]["kernel_launches"]
    for prec, res in results.items():
        q = step_bytes(prec, 4, res["mean_vcycles_per_solve"], krylov=res.get("krylov", False))
        sr = {"bytes_per_cell_step": q, "achieved": q * res["value"] / world / 1e9, "peak": peak, "unit": "GB/s",
              "peak_kind": peak_kind}
        sr["frac"] = sr["achieved"] / peak
        (out if prec == main_prec else out["mixed"])["step_roofline"] = sr
    if a.accuracy_steps > 0 and len(results) == 2:
        out["mixed"]["accuracy"] = accuracy(n, a.accuracy_steps)
    if rank == 0 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(n, 1)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
