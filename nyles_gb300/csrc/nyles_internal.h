// Internal (C++) interface between the translation units of libnyles_gb300.so.
// Nothing here crosses the public C ABI (include/nyles_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "nyles_common.cuh"
#include "../../include/nyles_gb300.h"

namespace nyles {

void set_error(const std::string& msg);
int cuda_status(cudaError_t e, const char* where);
void note_launch(int n = 1);

// CUDA-event profiler of the model phases (NYLES_NPHASE in the public header)
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> ev;   // 2 per slot
    std::vector<int> phase;
    size_t used = 0;
    double ms[NYLES_NPHASE] = {};
    long long cnt[NYLES_NPHASE] = {};
    int begin(int ph, cudaStream_t st);
    void end(int slot, cudaStream_t st);
    void flush();
    void release();
};
// RAII bracket of one phase; inert when the profiler is off or absent
struct ProfScope {
    Prof* p;
    int slot;
    cudaStream_t st;
    ProfScope(Prof* p_, int ph, cudaStream_t s) : p(p_), slot(-1), st(s) {
        if (p && p->on) slot = p->begin(ph, st);
    }
    ~ProfScope() {
        if (p && slot >= 0) p->end(slot, st);
    }
};

// Build the array geometry of a descriptor. Returns false on bad arguments.
bool make_geom(const NylesDesc* d, Geom* g);

template <typename T>
struct StencilPtrs {
    T* f[NYLES_F_T0 + NYLES_MAX_TR];   // state fields by NYLES_F_* id
};
template <typename T>
struct ProgPtrs {
    T* p[NYLES_MAX_PROG];              // prognostic registers: b, u_i, u_j, u_k, t0..
};

// term bits of launch_rhs
enum { TERM_TRACER = 1, TERM_VF = 2, TERM_BERNOULLI = 4, TERM_VISC = 8, TERM_ACCUMULATE = 16, TERM_TRDIFF = 32 };

// interior = true skips the b and u tendencies of periodic halo cells (the time step
// refills those halos before it reads them); false covers every stored cell
// `bat` (every launch_* below): a batched launch over the runs of its table (default:
// one run)
template <typename T>
int launch_rhs(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, const ProgPtrs<T>& ds, int terms,
               cudaStream_t st, bool interior = false, const Bat& bat = Bat());

// time-scheme elementwise updates (core/timescheme.py:113-221)
enum { UPD_EULER = 0, UPD_RK3_2 = 1, UPD_RK3_3 = 2, UPD_LF_PRED = 3, UPD_LF_FIRST = 4, UPD_LF_CORR = 5 };
template <typename T>
int launch_update(const Geom& g, int nprog, const ProgPtrs<T>& s, const ProgPtrs<T>& a, const ProgPtrs<T>& b,
                  const ProgPtrs<T>& c, int kind, double dt, cudaStream_t st, const Bat& bat = Bat());

template <typename T>
int launch_fill(const Geom& g, T* const* fields, int nf, cudaStream_t st, const Bat& bat = Bat());

// divergence of the contravariant velocity: writes state div (every cell, halo as its
// periodic image) and the interior right-hand side of the pressure solve
template <typename T, typename TB>
int launch_div(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, TB* mg_b, cudaStream_t st);

// projection correction of the interior velocity and p on every cell
template <typename T, typename TP>
int launch_correct(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, const TP* mg_x, double dx2,
                   cudaStream_t st);
// mixed precision: divergence into a float-pair right-hand side, correction from a
// float-pair solution
int launch_div_df(const NylesDesc* d, const Geom& g, const StencilPtrs<float>& s, float2* mg_b, cudaStream_t st,
                  const Bat& bat = Bat());
int launch_correct_df(const Geom& g, const StencilPtrs<float>& s, const float2* mg_x, double dx2, cudaStream_t st,
                      const Bat& bat = Bat());

// contravariant velocity, vorticity and kinetic energy from the filled velocity
template <typename T>
int launch_diag(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, int nonlinear, cudaStream_t st,
                const Bat& bat = Bat());

template <typename T>
int launch_flux1d(const T* u, const T* q, T* flux, int nlines, int n, cudaStream_t st);

template <typename T>
int launch_max_U2(const Geom& g, const StencilPtrs<T>& s, double* partial, int npartial, double* out,
                  cudaStream_t st);

// half-open index box of the (z, y, x) arrays summed by the vortex-force work diagnostic
struct VfBox {
    int lo[3], hi[3];
};
// work field of the vortex force held in ds.p[1..3] (u components), and its sum over box
template <typename T>
int launch_vfwork(const Geom& g, const StencilPtrs<T>& s, const ProgPtrs<T>& ds, const VfBox& box, double* partial,
                  int npartial, double* out, cudaStream_t st);

// ------------------------------------------------------------------ multigrid
struct MgLevelDesc {
    int n[3];         // interior extents z, y, x
    long long vol;
    size_t off_x, off_b, off_y;   // byte offsets inside the workspace
};

struct MgImpl {
    int nlevels = 0;
    int per[3] = {0, 0, 0};
    int precision = NYLES_FP64;
    double tol = 1e-6, omega = 0.9;
    int maxite = 20;
    MgLevelDesc lev[32];
    int bottom = 0;                   // first level of the one-block coarse solve (nlevels: none)
    size_t bottom_smem = 0;           // its shared memory bytes
    // mixed precision: level-1 solution and right-hand side as float pairs (hi, lo);
    // `nsol` solution arrays one after the other (sol_bytes apart), `cur_sol` the one the
    // next solve starts from and updates (a model keeps one per stage of its time scheme)
    size_t off_pdf = 0, off_bdf = 0;
    int nsol = 1, cur_sol = 0;
    size_t sol_bytes = 0;
    // `nhist` (0..3): behind the nsol solutions, nhist x nsol more arrays holding the
    // solutions before each one, and per solution a count (0..4) of the solves it has
    // seen; with `extrap` p (1..nhist) a solve starts from the degree-p extrapolation
    int nhist = 0;
    int extrap = 0;
    size_t off_hist = 0;
    // mixed precision, Krylov acceleration (FCG(1) preconditioned by the V-cycle): the
    // search direction and its image under the operator, level-1 floats
    int krylov = 0;
    size_t off_fp = 0, off_fq = 0;
    int fcg_k = 0;                    // iteration of the V-cycle being enqueued (-1: read on the device)
    // 4-cell vector kernels where the level-1 extents allow (off with the environment
    // variable NYLES_GB300_SCALAR_KERNELS=1, read when the solver is created)
    bool vec4 = true;
    // z-chunk of the vector kernels below level 0 (cells per thread along z: 1, 2 or 4;
    // NYLES_GB300_COARSE_ZC, read when the solver is created); level 0 keeps 4
    int czc = 1;
    // the ticket counter of reductions finished by their kernel's last block (MgFin)
    size_t off_ticket = 0;
    size_t off_partial = 0, off_partial2 = 0, off_scalars = 0;
    int npartial = 0;
    size_t bytes = 0;
    char* ws = nullptr;
    NylesMgStats stats{};
    Prof* prof = nullptr;             // phase timing (owned by the model)
    Bat bat;                          // batched launches (set while a batched step is captured)
};

int mg_init(MgImpl* mg, int nx, int ny, int nz, int topology, int precision, int nsol = 1, int nhist = 0);
// the float-pair level-1 solution the next mixed-precision solve works on
float2* mg_pdf(MgImpl* mg);
// forget the solutions kept for extrapolated warm starts (the next solves start plain)
int mg_reset_history(MgImpl* mg);
int mg_solve(MgImpl* mg, cudaStream_t st);
void* mg_level_ptr(MgImpl* mg, int lev, int var);

// Incremental construction of a CUDA graph from captured segments. Between segments
// the caller may add nodes by hand (conditional loops); `deps` is the frontier the next
// segment depends on.
struct GraphBuilder {
    cudaGraph_t graph = nullptr;
    cudaStream_t st = nullptr;
    std::vector<cudaGraphNode_t> deps;
    int error = 0;
    long long body_kernels = 0; // kernel launches captured in the last multigrid loop body
    void begin_segment();
    void end_segment();
};

// multigrid solve recorded into a graph: stop test on the device, V-cycles in a
// conditional while-node (solvers.f90:8-33)
int mg_solve_graph(MgImpl* mg, GraphBuilder& gb);
// device-side statistics of graph-mode solves: last nite, last res, and the totals of
// V-cycles, of solves stopped at maxite above tol and of solves stopped by a
// non-finite norm
struct MgDeviceStats {
    int nite = 0;
    double res = 0.0;
    long long vcycles = 0, not_converged = 0, nonfinite = 0;
};
int mg_read_device_stats(MgImpl* mg, cudaStream_t st, MgDeviceStats* out);
// zero the solver's device scalars (synchronous; at workspace binding)
int mg_zero_scalars(MgImpl* mg);

}  // namespace nyles
