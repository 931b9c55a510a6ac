/* nyles_gb300.h — C ABI of libnyles_gb300.so, the GB300 (sm_103a) implementation of
 * the Nyles LES time step for one subdomain on one GPU.
 *
 * Conventions
 *  - Plain C types only. Device arrays are raw pointers to row-major (z, y, x) arrays,
 *    the layout of the reference's `Scalar.view('i')` (core/variables.py:146-151),
 *    with an `nh`-cell halo on both sides of each periodic direction and none in
 *    closed directions (core/mpi/topology.py:253-300).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Every entry point returns an NYLES_* status; nyles_last_error() gives the message.
 *    Nothing calls exit(), traps, or asserts on the device.
 *  - The library never allocates device memory: the caller provides every array and a
 *    workspace whose size the library reports.
 *  - `_f64` entry points compute in double precision, `_f32` in single precision.
 */
#ifndef NYLES_GB300_H
#define NYLES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum {
    NYLES_OK = 0,
    NYLES_BAD_ARG = 1,
    NYLES_CUDA_ERROR = 2,
    NYLES_NOT_CONVERGED = 3, /* multigrid stopped at maxite above tolerance */
    NYLES_BLOWUP = 4,        /* a non-finite value reached the state */
    NYLES_TIMEOUT = 5,
    NYLES_UNSUPPORTED = 6
};

/* ---------------------------------------------------------------- enumerations */
/* core/nyles.py:92-100; NYLES_MODEL_ADVECTION is core/model_advection.py (b advected by
 * the stored contravariant velocity U, which the model never changes) */
enum { NYLES_MODEL_LES = 0, NYLES_MODEL_EULER3D = 1, NYLES_MODEL_LINEAR = 2, NYLES_MODEL_ADVECTION = 3 };
enum { NYLES_SCHEME_EF = 0, NYLES_SCHEME_LFAM3 = 1, NYLES_SCHEME_RK3_SSP = 2 };  /* core/timescheme.py:80-90 */
enum { NYLES_FP64 = 0, NYLES_MIXED = 1 };
/* multigrid topology, core/mgfor/mg_enums.f90:6 */
enum { NYLES_MG_CLOSED = 1, NYLES_MG_XPERIO = 2, NYLES_MG_YPERIO = 3, NYLES_MG_ZPERIO = 4,
       NYLES_MG_XYPERIO = 5, NYLES_MG_XYZPERIO = 6 };

/* state fields, in the table-of-contents order of core/variables.py:38-47;
 * tracer t<k> is NYLES_F_T0 + k (core/model_les.py:36-44) */
enum {
    NYLES_F_B = 0, NYLES_F_P = 1, NYLES_F_KE = 2, NYLES_F_DIV = 3,
    NYLES_F_U_I = 4, NYLES_F_U_J = 5, NYLES_F_U_K = 6,      /* covariant velocity u */
    NYLES_F_UC_I = 7, NYLES_F_UC_J = 8, NYLES_F_UC_K = 9,   /* contravariant velocity U */
    NYLES_F_VOR_I = 10, NYLES_F_VOR_J = 11, NYLES_F_VOR_K = 12,
    NYLES_F_WORK = 13, NYLES_F_T0 = 14
};
#define NYLES_MAX_TRACERS 8
/* prognostic registers (core/variables.py:364-383 order): b, u_i, u_j, u_k, t0.. */

/* ---------------------------------------------------------------- descriptors */
typedef struct NylesDesc {
    int nx, ny, nz;          /* interior cells of the subdomain (param nx, ny, nz) */
    int nh;                  /* halo width of periodic directions (param nh) */
    int periodic_x, periodic_y, periodic_z;   /* from param geometry */
    int n_tracers;           /* param n_tracers */
    int model;               /* NYLES_MODEL_* */
    int add_viscosity;       /* 1 when diff_coef has 'u' */
    double dx, dy, dz;       /* grid spacing, core/grid.py:30-32 */
    double idx2, idy2, idz2; /* 1/dx**2 etc. as computed by the host, core/grid.py:38-40 */
    double dx2;              /* dx**2 as computed by the host, core/mgfordriver.py:78 */
    double fparam;           /* covariant Coriolis coriolis*dx*dy (0 when not rotating), core/model_les.py:61-67 */
    double viscosity;        /* diff_coef['u'], core/viscosity.py:3-9 */
    /* Tracer diffusion (core/tracer.py:74-76): diff_coef of b, t0, t1.. added as
     * add_laplacian after each direction's advection on the last stage. The reference
     * never passes `last` to rhstrac (core/model_les.py:133), so its tracer diffusion
     * never runs; it runs here only when bit q of tracer_diffusion is set (q = 0 for b,
     * 1 + k for tk). 0 = the reference's behaviour. */
    double tracer_diffusivity[NYLES_MAX_TRACERS + 1];
    int tracer_diffusion;
    /* Tracer advection scheme: 0 = WENO (core/fortran_upwind.f90:63-80, the only branch
     * the reference runs: `linear` is hard-coded .false. at :28); 1..5 = the linear
     * branch of core/fortran_upwind.f90:32-61 with the interpolation of that order
     * from core/interpolate_tracer.f90 (odd: upwind-biased, even: centred), i.e.
     * param orderA. */
    int tracer_order;
    /* Vortex-force reconstruction: 0 = WENO (core/fortran_vortex_force.f90:56-82 and
     * :134-160, the only branch the reference runs: `linear` is hard-coded .false. at
     * :28 and :106); 1..5 = the linear branch of :43-55 (direc) and :121-133 (flip)
     * with core/interpolate.f90:3-112 of that order (odd: upwinded with the split
     * velocity; even: the interpolated vorticity alone, as written there), i.e. param
     * orderVF. */
    int vf_order;
} NylesDesc;

typedef struct NylesMgStats {
    int nite;          /* V-cycles of the last solve (mgfor MG_Stats%nite) */
    double res;        /* last squared residual ratio sum(r^2)/sum(b^2) (mgfor MG_Stats%res) */
    long long solves;  /* solves since creation */
    long long vcycles; /* V-cycles since creation */
    int not_converged; /* solves that stopped at maxite above tol */
    int nonfinite;     /* solves stopped by a non-finite norm of b or of a residual (blow-up) */
} NylesMgStats;

const char* nyles_last_error(void);
int nyles_version(void);

/* ---------------------------------------------------------------- kernels
 * One-dimensional upwind flux with WENO5/WENO3 reconstruction and the reference's
 * boundary closures, on `nlines` independent lines of length n (n >= 5), lines
 * contiguous. Replaces core/weno.f90:106-153 (flux1d). */
int nyles_flux1d_f64(const double* u, const double* q, double* flux, int nlines, int n, void* stream);
int nyles_flux1d_f32(const float* u, const float* q, float* flux, int nlines, int n, void* stream);

/* Vortex force, added into the velocity registers ds[1..3]:
 * du_i += -(omega x U)_i with omega upwinded along the advecting direction.
 * Replaces core/vortex_force.py:14-81 -> core/fortran_vortex_force.f90:10-165
 * (vortex_force_direc / vortex_force_flip, six calls). `fields` indexed by NYLES_F_*. */
int nyles_vortex_force_f64(const NylesDesc* d, double* const* fields, double* const* ds, void* stream);
int nyles_vortex_force_f32(const NylesDesc* d, float* const* fields, float* const* ds, void* stream);

/* Right-hand side of the model into registers ds (overwritten, as reset_state):
 * tracer flux divergence (core/tracer.py:44-78 -> fortran_upwind.f90:3-87), vortex
 * force, Bernoulli (core/bernoulli.py:14-32 -> fortran_bernoulli.f90:2-58) and, when
 * `last` and add_viscosity, viscosity (core/viscosity.py:3-9 -> fortran_dissipation.f90:2-35).
 * Replaces core/model_les.py:130-144 (LES.rhs) and core/model_les_euler.py:128-142. */
int nyles_rhs_f64(const NylesDesc* d, double* const* fields, double* const* ds, int last, void* stream);
int nyles_rhs_f32(const NylesDesc* d, float* const* fields, float* const* ds, int last, void* stream);

/* Periodic halo fill of one field. Replaces core/mpi/halo.py:140-178 (Halo.fill) for one rank. */
int nyles_fill_f64(const NylesDesc* d, double* field, void* stream);
int nyles_fill_f32(const NylesDesc* d, float* field, void* stream);

/* ---------------------------------------------------------------- multigrid
 * Cell-centred geometric multigrid of one rank. Replaces the ctypes interface of
 * core/mgfordriver.py:6-105 over core/mgfor: get_ptrmg (mg_setup.f90:318-437),
 * get_pyshape/set_pyarray/get_pyarray (pytools.f90:8-60), solve (solvers.f90:8-33).
 * Level arrays hold interior cells only, (nz, ny, nx) row-major; ghost layers of the
 * reference are implied (zero across closed walls, periodic image otherwise).
 * precision NYLES_MIXED: FP32 V-cycles inside FP64 iterative refinement. */
typedef struct NylesMg NylesMg;
int nyles_mg_create(int nx, int ny, int nz, int topology, int precision, NylesMg** out);
int nyles_mg_destroy(NylesMg* mg);
int nyles_mg_workspace_bytes(const NylesMg* mg, size_t* bytes);
int nyles_mg_bind(NylesMg* mg, void* workspace);      /* device memory of workspace_bytes */
int nyles_mg_nlevels(const NylesMg* mg, int* nlevels);
int nyles_mg_level_shape(const NylesMg* mg, int lev, int* shape3); /* lev 1 = finest */
/* var 1 = x (solution), 2 = b (right-hand side). Elements are double (NYLES_FP64) or
 * float (NYLES_MIXED), except lev 1 in NYLES_MIXED: interleaved float pairs (hi, lo)
 * whose value is hi + lo, |lo| <= ulp(hi)/2. */
int nyles_mg_level_ptr(NylesMg* mg, int lev, int var, void** ptr);
/* tol on the squared residual ratio (mg_types.f90:15-26; defaults 1e-6, 20, 0.9) */
int nyles_mg_set_params(NylesMg* mg, double tol, int maxite, double omega);
/* Mixed precision only: with on = 1 the solve is flexible conjugate gradients (FCG(1))
 * on the level-1 equation, preconditioned by one FP32 V-cycle per iteration, with the
 * float-pair solution and the float-pair true residual of the stop test (same rule:
 * sum(r^2)/sum(b^2) < tol or maxite iterations). It reaches a tight tolerance in about
 * half the V-cycles of the reference's stationary iteration (mgfor solvers.f90:8-33),
 * whose iterates it no longer follows; 0 (default) keeps that iteration.
 * NYLES_UNSUPPORTED for an FP64 solver. */
int nyles_mg_set_krylov(NylesMg* mg, int on);
/* NYLES_NOT_CONVERGED when it stopped at maxite above tol; NYLES_BLOWUP, at once, when
 * the norm of the right-hand side or of a residual is not finite */
int nyles_mg_solve(NylesMg* mg, NylesMgStats* stats, void* stream);

/* ---------------------------------------------------------------- whole model
 * One subdomain of LES / Euler3d / linear (core/nyles.py:92-100) with its time scheme
 * and pressure projection. The caller owns every array:
 *   fields   : NYLES_F_T0 + n_tracers device pointers (NYLES_F_* order)
 *   regs     : 3 * (4 + n_tracers) device pointers, register r of prognostic q at
 *              regs[r*(4+n_tracers)+q] (RK3: ds0, ds1, ds2; LFAM3: dstate, stateb,
 *              state; EF: dstate), core/timescheme.py:92-101
 *   workspace: nyles_model_workspace_bytes() bytes of device memory
 * precision NYLES_FP64: double arrays; NYLES_MIXED: float arrays (FP64 pressure). */
typedef struct NylesModel NylesModel;
int nyles_model_create(const NylesDesc* d, int scheme, int precision, NylesModel** out);
int nyles_model_destroy(NylesModel* m);
int nyles_model_workspace_bytes(const NylesModel* m, size_t* bytes);
int nyles_model_bind(NylesModel* m, void* const* fields, void* const* regs, void* workspace);
int nyles_model_set_mg_params(NylesModel* m, double tol, int maxite, double omega);
/* nyles_mg_set_krylov for the model's pressure solve (refused while a graph is captured) */
int nyles_model_set_mg_krylov(NylesModel* m, int on);
/* Warm start of the pressure solves. 0 (default): every solve starts from the last
 * solve's solution, as the reference's single mgfor x does (core/mgfordriver.py:66-78).
 * 1, mixed precision only: the k-th projection of a step starts from the solution of
 * the k-th projection of the previous step (one float-pair solution per projection of
 * the time scheme). The stages of a step project divergences of different tendency
 * combinations, so the same stage one step earlier is the nearer start. 2, mixed
 * precision only: as 1, from the linear extrapolation 2 x(n-1) - x(n-2) of the same
 * stage's last two solutions (once it has two). 3: the quadratic extrapolation
 * 3 x(n-1) - 3 x(n-2) + x(n-3) once it has three (linear with two); 4: the cubic one
 * 4 x(n-1) - 6 x(n-2) + 4 x(n-3) - x(n-4) once it has four. The solution is
 * the same to the solve's tolerance, in fewer V-cycles. No counterpart in the
 * reference. The mode sizes the workspace (mode m > 0 keeps nstage x (1 + max(0, m-1))
 * float-pair solutions of the fine level): select it before
 * nyles_model_workspace_bytes and nyles_model_bind; a bound model accepts only modes
 * whose arrays its workspace holds (else NYLES_BAD_ARG). Changing the mode forgets the
 * kept solutions.
 * NYLES_UNSUPPORTED for an FP64 model (its parity keeps the reference's). */
int nyles_model_set_mg_warm_start(NylesModel* m, int mode);
/* LES.forward: one time step, core/model_les.py:147-149 -> core/timescheme.py:113-221.
 * Returns NYLES_BLOWUP when a pressure solve of the step meets a non-finite divergence
 * (a non-finite velocity, or a buoyancy that reached the velocity): the step stops at
 * that stage and leaves the state as it is. Other non-finite values are caught by
 * nyles_model_max_U2. */
int nyles_model_forward(NylesModel* m, double t, double dt, void* stream);
/* LES.diagnose_var, core/model_les.py:98-127 (core/model_les_euler.py:96-125) */
int nyles_model_diagnose(NylesModel* m, void* stream);
/* LES.rhs(state, t, dstate, last) into register set `reg`, core/model_les.py:130-144
 * (advection model: Advection.rhs, core/model_advection.py:59-61, b only; the velocity
 * registers are left as they are) */
int nyles_model_rhs(NylesModel* m, int reg, double t, int last, void* stream);
/* Advection.make_u_divergentfree, core/model_advection.py:38-53: fill u, project u with
 * the multigrid (p = x*dx^2, u -= grad p, as LES.diagnose_var), fill u, U = u/dx^2 and
 * div of the new U (halo filled). Any model kind. */
int nyles_model_project(NylesModel* m, void* stream);
/* User forcing (core/model_les.py:143-144, `forcing.add(state, dstate, t)` when the
 * parameter `forced` is set): `fn(user, reg, t, stream)` is called on the host after
 * every right-hand side of forward/rhs, with the register set holding that stage's
 * tendencies and the stage time (RK3: t, t + dt, t + dt/2; LFAM3: t, t + dt/2; EF: t);
 * it adds its tendencies by work enqueued on `stream`. NULL detaches it. A model with
 * a forcing cannot be captured into a graph. */
typedef void (*nyles_forcing_fn)(void* user, int reg, double t, void* stream);
int nyles_model_set_forcing(NylesModel* m, nyles_forcing_fn fn, void* user);
/* max over the arrays of U^2+V^2+W^2 (core/nyles.py:241-251), copied to *out */
int nyles_model_max_U2(NylesModel* m, double* out, void* stream);
/* VFwork.compute, core/online_diag.py:11-35: the u components of register set 0 are
 * zeroed and receive the vortex force alone, the work field NYLES_F_WORK gets
 * sum_d (U_d F_d / 2)(p) + (U_d F_d / 2)(p - e_d), and *worksum its sum (FP64) over the
 * half-open box {z0, z1, y0, y1, x0, x1} of the arrays. Synchronises `stream`. */
int nyles_model_vfwork(NylesModel* m, const long long* box, double* worksum, void* stream);
int nyles_model_mg_stats(const NylesModel* m, NylesMgStats* stats);
/* a fresh LFAM3 start (its first step is Euler forward, core/timescheme.py:129-140) */
int nyles_model_reset_scheme(NylesModel* m);
/* LFAM3's `first` flag (core/timescheme.py:94, the Euler first step still to take),
 * read and restored with a snapshot of the device state. No counterpart in the
 * reference (its LFAM3 state is not checkpointable). */
int nyles_model_get_first_step(const NylesModel* m, int* pending);
int nyles_model_set_first_step(NylesModel* m, int pending);

/* CUDA-graph replay of nsteps time steps of LES.forward with a fixed dt (no counterpart
 * in the reference, whose step is a Python loop). The multigrid stop test runs on the
 * device (a conditional while-node per pressure solve), so one launch advances nsteps
 * steps with no host synchronisation; results equal nyles_model_forward's. LFAM3 must
 * have taken its first (Euler) step before capture. nyles_model_mg_stats reads the
 * device-side statistics after launches. */
int nyles_model_capture(NylesModel* m, double dt, int nsteps);
int nyles_model_graph_launch(NylesModel* m, void* stream);
int nyles_model_graph_release(NylesModel* m);

/* ---------------------------------------------------------------- batched steps
 * No counterpart in the reference (one experiment per process, core/nyles.py:44-117).
 * A bucket of runs with the same grid, precision and parameters advances with one
 * graph launch: every kernel of the recorded steps covers up to nrun runs. Each run's
 * memory (its fields, registers and workspace, in one allocation laid out as the
 * model's own) lies delta[r] bytes from the memory the model was bound to; slot r is
 * advanced when active[r] is nonzero, and its pressure solves stop on their own
 * (live[r], written on the device), so a run's result does not depend on the others.
 * The caller writes delta and active into the device table before each launch;
 * loop_iterations counts the multigrid loop-body iterations run (device-side). */
#define NYLES_BATCH_RUNS 32
typedef struct NylesBatchTable {
    long long delta[NYLES_BATCH_RUNS];  /* byte distance of run r's memory from the model's */
    int active[NYLES_BATCH_RUNS];       /* 1: slot r holds a run that the launch advances */
    int live[NYLES_BATCH_RUNS];         /* device-side: run r's current solve still iterates */
    long long loop_iterations;          /* device-side: multigrid loop-body iterations run */
} NylesBatchTable;
/* Record nsteps steps with a fixed dt (nsteps = 0: one LES.diagnose_var, the initial
 * projection of a run, core/model_les.py:98-127) for nrun (<= NYLES_BATCH_RUNS) runs
 * whose table is the device memory `table`, into a new batched graph. The graph refers
 * to m's memory (shifted per run by the table); m must stay bound while it is launched.
 * Mixed-precision LES with the stationary pressure solve, no tracers, the reference's
 * schemes; NYLES_UNSUPPORTED otherwise. */
typedef struct NylesBatchGraph NylesBatchGraph;
int nyles_model_batch_capture(NylesModel* m, double dt, int nsteps, int nrun, NylesBatchTable* table,
                              NylesBatchGraph** out);
int nyles_batch_launch(NylesBatchGraph* g, void* stream);
/* adds the kernels of `iterations` multigrid loop-body iterations (read from the table)
 * to nyles_launch_count */
int nyles_batch_note_iterations(const NylesBatchGraph* g, long long iterations);
int nyles_batch_destroy(NylesBatchGraph* g);
/* The counters the pressure solves of recorded (graph or batched) steps keep on the
 * device, read from the model's workspace: last nite and res, V-cycles, solves stopped
 * at maxite above tol, solves stopped by a non-finite norm (solves = 0). Synchronises
 * `stream`. */
int nyles_model_device_stats(NylesModel* m, NylesMgStats* stats, void* stream);

/* ---------------------------------------------------------------- instrumentation
 * No counterpart in the reference (its timing is core/timing.py's wall-clock decorator).
 * Phases: 0 right-hand side, 1 time-scheme update, 2 halo fill, 3 divergence,
 * 4 multigrid solve, 5 projection correction, 6 vorticity/ke/U, 7 CFL reduction,
 * 8 multigrid smoothing, 9 multigrid residual+restriction, 10 multigrid prolongation,
 * 11 multigrid norms. Profiling brackets each phase with CUDA events on the launching
 * stream (no host synchronisation added). */
#define NYLES_NPHASE 12
int nyles_model_profile(NylesModel* m, int enable);
/* per-phase device milliseconds and counts since enable (or last read); resets them */
int nyles_model_profile_read(NylesModel* m, double* ms, long long* count, int nphase);
/* number of kernels this library has launched in the process */
long long nyles_launch_count(void);

/* ---------------------------------------------------------------- allocation-free CFL reduction
 * No counterpart in the reference. Same result as nyles_model_max_U2 (the maximum over
 * n cells of U^2+V^2+W^2, core/nyles.py:241-251), written to *out, a device double,
 * without a model, a workspace or any allocation. It is meant for callers that cannot
 * allocate device memory: a host framework that owns every device allocation through a
 * pre-sized pool, a time loop that must not allocate between steps, a caller reaching
 * this library through a plain C or ctypes binding with no allocator of its own.
 * The reduction's block partials live in a static device array of NYLES_STATIC_PARTIALS
 * doubles (8 KiB, held by every GPU that loads the library until the process exits).
 * n is limited to NYLES_STATIC_MAX_CELLS; larger n returns NYLES_BAD_ARG.
 * The array's device address belongs to the current context: every call made outside
 * stream capture looks it up afresh, with the calling device current, and records it for
 * that device; a call made while `stream` is capturing reuses the address recorded by the
 * last call outside capture on the device (NYLES_BAD_ARG when there was none). So make
 * the first call on a device before any stream capture, and make one more outside
 * capture after a cudaDeviceReset or any re-creation of the device's primary context,
 * before capturing again. Every call writes the partials it reads, so nothing carries
 * over from one call to the next; but calls share the array, so calls that overlap on
 * the GPU (different streams or threads) race. */
#define NYLES_STATIC_PARTIALS 1024
#define NYLES_STATIC_MAX_CELLS (1LL << 28)
int nyles_max_U2_static_f64(const double* U, const double* V, const double* W, long long n, double* out,
                            void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NYLES_GB300_H */
