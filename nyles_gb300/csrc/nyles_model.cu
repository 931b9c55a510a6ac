// C ABI of libnyles_gb300.so and the native orchestration of one time step
// (core/model_les.py, core/model_les_euler.py, core/timescheme.py, core/projection.py,
// core/mgfordriver.py restated as a sequence of kernel launches on one stream).
#include "nyles_internal.h"
#include <atomic>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>

namespace nyles {

static_assert(sizeof(BatchTab) == sizeof(NylesBatchTable) && offsetof(BatchTab, active) == offsetof(NylesBatchTable, active) &&
                  offsetof(BatchTab, live) == offsetof(NylesBatchTable, live) &&
                  offsetof(BatchTab, loop_iterations) == offsetof(NylesBatchTable, loop_iterations) &&
                  NYLES_MAX_BATCH == NYLES_BATCH_RUNS,
              "the device batch table and NylesBatchTable of the public header differ");

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return NYLES_OK;
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return NYLES_CUDA_ERROR;
}

static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// ------------------------------------------------------------------ profiler
static const size_t kProfSlots = 4096;

int Prof::begin(int ph, cudaStream_t st) {
    if (ev.empty()) {
        ev.resize(2 * kProfSlots);
        phase.resize(kProfSlots);
        for (auto& e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) { ev.clear(); on = false; return -1; }
    }
    if (used == kProfSlots) flush();
    const int slot = (int)used++;
    phase[slot] = ph;
    cudaEventRecord(ev[2 * slot], st);
    return slot;
}

void Prof::end(int slot, cudaStream_t st) { cudaEventRecord(ev[2 * slot + 1], st); }

void Prof::flush() {
    if (used == 0) return;
    cudaEventSynchronize(ev[2 * (used - 1) + 1]);
    for (size_t s = 0; s < used; ++s) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ev[2 * s], ev[2 * s + 1]) == cudaSuccess) {
            ms[phase[s]] += t;
            cnt[phase[s]] += 1;
        }
    }
    used = 0;
}

void Prof::release() {
    for (auto& e : ev) cudaEventDestroy(e);
    ev.clear();
    used = 0;
}

static int check_desc(const NylesDesc* d, Geom* g) {
    if (!d) { set_error("null descriptor"); return NYLES_BAD_ARG; }
    if (d->n_tracers < 0 || d->n_tracers > NYLES_MAX_TR) { set_error("n_tracers out of range (0..8)"); return NYLES_BAD_ARG; }
    if (d->model < 0 || d->model > 3) { set_error("unknown model"); return NYLES_BAD_ARG; }
    if (d->model == NYLES_MODEL_ADVECTION && d->n_tracers != 0) {
        set_error("the advection model advects b only (n_tracers must be 0)");
        return NYLES_BAD_ARG;
    }
    if (d->tracer_order < 0 || d->tracer_order > 5) {
        set_error("tracer_order must be 0 (WENO) or an interpolation order 1..5");
        return NYLES_BAD_ARG;
    }
    if (d->vf_order < 0 || d->vf_order > 5) {
        set_error("vf_order must be 0 (WENO) or an interpolation order 1..5");
        return NYLES_BAD_ARG;
    }
    if (d->tracer_diffusion < 0 || (d->tracer_diffusion >> (d->n_tracers + 1)) != 0) {
        set_error("tracer_diffusion names a tracer beyond b, t0..t{n_tracers-1}");
        return NYLES_BAD_ARG;
    }
    if ((d->periodic_x || d->periodic_y || d->periodic_z) && d->nh != 3) {
        set_error("periodic directions need nh == 3 (the multigrid halo width, mg_types.f90:18)");
        return NYLES_UNSUPPORTED;
    }
    if (!make_geom(d, g)) { set_error("bad grid extents (every array line needs at least 5 points)"); return NYLES_BAD_ARG; }
    return NYLES_OK;
}

template <typename T>
static StencilPtrs<T> field_ptrs(const NylesDesc* d, T* const* fields) {
    StencilPtrs<T> s;
    for (int i = 0; i < NYLES_F_T0 + NYLES_MAX_TR; ++i)
        s.f[i] = (i < NYLES_F_T0 + d->n_tracers) ? fields[i] : nullptr;
    return s;
}
template <typename T>
static ProgPtrs<T> prog_ptrs(const NylesDesc* d, T* const* p) {
    ProgPtrs<T> s;
    for (int i = 0; i < NYLES_MAX_PROG; ++i) s.p[i] = (p && i < 4 + d->n_tracers) ? p[i] : nullptr;
    return s;
}
template <typename T>
static ProgPtrs<T> state_prog(const NylesDesc* d, const StencilPtrs<T>& s) {
    ProgPtrs<T> p;
    for (int i = 0; i < NYLES_MAX_PROG; ++i) p.p[i] = nullptr;
    p.p[0] = s.f[NYLES_F_B];
    for (int k = 0; k < 3; ++k) p.p[1 + k] = s.f[NYLES_F_U_I + k];
    for (int t = 0; t < d->n_tracers; ++t) p.p[4 + t] = s.f[NYLES_F_T0 + t];
    return p;
}

static int rhs_terms(const NylesDesc* d, int last) {
    // Advection.rhs passes `last` to rhstrac, so its diffusion of b is live
    // (core/model_advection.py:59-61)
    if (d->model == NYLES_MODEL_ADVECTION) return TERM_TRACER | ((last && (d->tracer_diffusion & 1)) ? TERM_TRDIFF : 0);
    int t = TERM_BERNOULLI;
    if (d->model != NYLES_MODEL_EULER3D) t |= TERM_TRACER;   // model_les_euler.py:131
    if (d->model != NYLES_MODEL_LINEAR) t |= TERM_VF;        // model_les.py:135-136
    if (last && d->add_viscosity) t |= TERM_VISC;            // model_les.py:140-141
    // tracer.py:74-76 (opt-in: the reference's rhs never passes last to rhstrac)
    if (last && d->tracer_diffusion && d->model != NYLES_MODEL_EULER3D) t |= TERM_TRDIFF;
    return t;
}

}  // namespace nyles

using namespace nyles;

struct NylesMg {
    MgImpl impl;
};

// A recorded batched graph: its executable and its kernel counts. It refers to the
// memory of the model it was recorded on, shifted per run through the table.
struct NylesBatchGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;        // per launch, outside the multigrid loops
    long long body_kernels = 0;   // per loop-body iteration
    ~NylesBatchGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

struct NylesModel {
    NylesDesc d;
    Geom g;
    int scheme = NYLES_SCHEME_RK3_SSP;
    int precision = NYLES_FP64;
    int topo = NYLES_MG_CLOSED;
    int nstage = 3;                      // projections per time step (RK3: 3, LFAM3: 2, EF: 1)
    int nprog = 4;
    bool lf_first = true;
    void* fields[NYLES_F_T0 + NYLES_MAX_TR] = {};
    void* regs[3][NYLES_MAX_PROG] = {};
    char* ws = nullptr;
    size_t off_partial = 0, off_scalar = 0, mg_off = 0, bytes = 0;
    int npartial = 152 * 4;
    MgImpl mg;
    Prof prof;
    bool bound = false;
    // graph mode: one or more captured time steps replayed with one launch
    GraphBuilder* gb = nullptr;          // set while capturing
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long graph_kernels = 0;         // kernels outside the multigrid loops per launch
    long long graph_body_kernels = 0;    // kernels per V-cycle iteration of a loop
    int graph_solves = 0;                // pressure solves per launch
    long long graph_launches = 0;
    long long vcycles_counted = 0;       // device V-cycles already added to the launch count
    bool last_solve_graph = false;       // the latest solve ran inside a graph
    cudaStream_t last_stream = nullptr;  // stream of the latest graph launch
    nyles_forcing_fn forcing = nullptr;  // user forcing called after each right-hand side
    void* forcing_user = nullptr;
    Bat bat;                             // set while a batched graph is recorded
    // mixed precision: each stage's pressure solve starts from the solution of the same
    // stage of the previous step (1) or, as the reference, from the last solve's (0)
    int warm_per_stage = 0;
    void release_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    }
    ~NylesModel() {
        prof.release();
        release_graph();
        if (cap_stream) cudaStreamDestroy(cap_stream);
    }
};

extern "C" {

const char* nyles_last_error(void) { return g_last_error.c_str(); }
int nyles_version(void) { return 10000; }

// ------------------------------------------------------------------ kernel entries
int nyles_flux1d_f64(const double* u, const double* q, double* flux, int nlines, int n, void* stream) {
    if (n < 5 || nlines < 0 || !u || !q || !flux) { set_error("flux1d: n >= 5 and non-null arrays required"); return NYLES_BAD_ARG; }
    return launch_flux1d<double>(u, q, flux, nlines, n, (cudaStream_t)stream);
}
int nyles_flux1d_f32(const float* u, const float* q, float* flux, int nlines, int n, void* stream) {
    if (n < 5 || nlines < 0 || !u || !q || !flux) { set_error("flux1d: n >= 5 and non-null arrays required"); return NYLES_BAD_ARG; }
    return launch_flux1d<float>(u, q, flux, nlines, n, (cudaStream_t)stream);
}

extern "C++" {
template <typename T>
static int vortex_force_impl(const NylesDesc* d, T* const* fields, T* const* ds, void* stream) {
    Geom g;
    int rc = check_desc(d, &g);
    if (rc) return rc;
    if (!fields || !ds) { set_error("null arrays"); return NYLES_BAD_ARG; }
    return launch_rhs<T>(d, g, field_ptrs<T>(d, fields), prog_ptrs<T>(d, ds), TERM_VF | TERM_ACCUMULATE,
                         (cudaStream_t)stream);
}
}  // extern "C++"
int nyles_vortex_force_f64(const NylesDesc* d, double* const* fields, double* const* ds, void* stream) {
    return vortex_force_impl<double>(d, fields, ds, stream);
}
int nyles_vortex_force_f32(const NylesDesc* d, float* const* fields, float* const* ds, void* stream) {
    return vortex_force_impl<float>(d, fields, ds, stream);
}

extern "C++" {
template <typename T>
static int rhs_impl(const NylesDesc* d, T* const* fields, T* const* ds, int last, void* stream) {
    Geom g;
    int rc = check_desc(d, &g);
    if (rc) return rc;
    if (!fields || !ds) { set_error("null arrays"); return NYLES_BAD_ARG; }
    return launch_rhs<T>(d, g, field_ptrs<T>(d, fields), prog_ptrs<T>(d, ds), rhs_terms(d, last),
                         (cudaStream_t)stream);
}
}  // extern "C++"
int nyles_rhs_f64(const NylesDesc* d, double* const* fields, double* const* ds, int last, void* stream) {
    return rhs_impl<double>(d, fields, ds, last, stream);
}
int nyles_rhs_f32(const NylesDesc* d, float* const* fields, float* const* ds, int last, void* stream) {
    return rhs_impl<float>(d, fields, ds, last, stream);
}

extern "C++" {
template <typename T>
static int fill_impl(const NylesDesc* d, T* field, void* stream) {
    Geom g;
    int rc = check_desc(d, &g);
    if (rc) return rc;
    if (!field) { set_error("null array"); return NYLES_BAD_ARG; }
    T* f[1] = {field};
    return launch_fill<T>(g, f, 1, (cudaStream_t)stream);
}
}  // extern "C++"
int nyles_fill_f64(const NylesDesc* d, double* field, void* stream) { return fill_impl<double>(d, field, stream); }
int nyles_fill_f32(const NylesDesc* d, float* field, void* stream) { return fill_impl<float>(d, field, stream); }

// ------------------------------------------------------------------ multigrid
int nyles_mg_create(int nx, int ny, int nz, int topology, int precision, NylesMg** out) {
    if (!out) { set_error("null output"); return NYLES_BAD_ARG; }
    *out = nullptr;
    if (precision != NYLES_FP64 && precision != NYLES_MIXED) { set_error("bad precision"); return NYLES_BAD_ARG; }
    NylesMg* m = new (std::nothrow) NylesMg();
    if (!m) { set_error("host allocation failed"); return NYLES_BAD_ARG; }
    int rc = mg_init(&m->impl, nx, ny, nz, topology, precision);
    if (rc) { delete m; return rc; }
    *out = m;
    return NYLES_OK;
}
int nyles_mg_destroy(NylesMg* mg) { delete mg; return NYLES_OK; }
int nyles_mg_workspace_bytes(const NylesMg* mg, size_t* bytes) {
    if (!mg || !bytes) { set_error("null argument"); return NYLES_BAD_ARG; }
    *bytes = mg->impl.bytes;
    return NYLES_OK;
}
int nyles_mg_bind(NylesMg* mg, void* workspace) {
    if (!mg || !workspace) { set_error("null argument"); return NYLES_BAD_ARG; }
    if (((uintptr_t)workspace) & 255) { set_error("workspace must be 256-byte aligned"); return NYLES_BAD_ARG; }
    mg->impl.ws = (char*)workspace;
    return mg_zero_scalars(&mg->impl);
}
int nyles_mg_nlevels(const NylesMg* mg, int* nlevels) {
    if (!mg || !nlevels) { set_error("null argument"); return NYLES_BAD_ARG; }
    *nlevels = mg->impl.nlevels;
    return NYLES_OK;
}
int nyles_mg_level_shape(const NylesMg* mg, int lev, int* shape3) {
    if (!mg || !shape3 || lev < 1 || lev > mg->impl.nlevels) { set_error("bad level"); return NYLES_BAD_ARG; }
    for (int k = 0; k < 3; ++k) shape3[k] = mg->impl.lev[lev - 1].n[k];
    return NYLES_OK;
}
int nyles_mg_level_ptr(NylesMg* mg, int lev, int var, void** ptr) {
    if (!mg || !ptr || var < 1 || var > 2) { set_error("bad argument"); return NYLES_BAD_ARG; }
    *ptr = mg_level_ptr(&mg->impl, lev, var);
    if (!*ptr) { set_error("workspace not bound or bad level"); return NYLES_BAD_ARG; }
    return NYLES_OK;
}
int nyles_mg_set_params(NylesMg* mg, double tol, int maxite, double omega) {
    if (!mg || maxite < 0 || !(tol >= 0.0) || !(omega > 0.0)) { set_error("bad multigrid parameters"); return NYLES_BAD_ARG; }
    mg->impl.tol = tol; mg->impl.maxite = maxite; mg->impl.omega = omega;
    return NYLES_OK;
}
static int set_krylov(MgImpl* mg, int on) {
    if (on && mg->precision != NYLES_MIXED) {
        set_error("Krylov acceleration is provided for the mixed-precision solve only (the FP64 solve keeps "
                  "the reference's iteration)");
        return NYLES_UNSUPPORTED;
    }
    mg->krylov = on ? 1 : 0;
    return NYLES_OK;
}
int nyles_mg_set_krylov(NylesMg* mg, int on) {
    if (!mg) { set_error("null multigrid"); return NYLES_BAD_ARG; }
    return set_krylov(&mg->impl, on);
}
int nyles_mg_solve(NylesMg* mg, NylesMgStats* stats, void* stream) {
    if (!mg) { set_error("null multigrid"); return NYLES_BAD_ARG; }
    int rc = mg_solve(&mg->impl, (cudaStream_t)stream);
    if (stats) *stats = mg->impl.stats;
    if (rc) return rc;
    return mg->impl.stats.nite >= mg->impl.maxite && mg->impl.stats.res >= mg->impl.tol ? NYLES_NOT_CONVERGED : NYLES_OK;
}

// ------------------------------------------------------------------ model
// Workspace layout: the multigrid (its level arrays; `nsol` float-pair solutions with
// `nhist` earlier solutions each in mixed precision), then partial sums and scalars.
// The warm start of nyles_model_set_mg_warm_start sets nsol and nhist before binding.
static int model_layout(NylesModel* m, int nsol, int nhist) {
    const NylesDesc* d = &m->d;
    int rc = mg_init(&m->mg, d->nx, d->ny, d->nz, m->topo, m->precision, nsol, nhist);
    if (rc) return rc;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    m->mg_off = take(m->mg.bytes);
    m->off_partial = take(m->npartial * sizeof(double));
    m->off_scalar = take(16 * sizeof(double));
    m->bytes = off;
    return NYLES_OK;
}

int nyles_model_create(const NylesDesc* d, int scheme, int precision, NylesModel** out) {
    if (!out) { set_error("null output"); return NYLES_BAD_ARG; }
    *out = nullptr;
    Geom g;
    int rc = check_desc(d, &g);
    if (rc) return rc;
    if (scheme < 0 || scheme > 2) { set_error("unknown time scheme"); return NYLES_BAD_ARG; }
    if (precision != NYLES_FP64 && precision != NYLES_MIXED) { set_error("bad precision"); return NYLES_BAD_ARG; }
    NylesModel* m = new (std::nothrow) NylesModel();
    if (!m) { set_error("host allocation failed"); return NYLES_BAD_ARG; }
    m->d = *d;
    m->g = g;
    m->scheme = scheme;
    m->precision = precision;
    m->nprog = 4 + d->n_tracers;
    // multigrid topology from the geometry (core/model_les.py:80-93)
    int topo;
    if (d->periodic_x && d->periodic_y && d->periodic_z) topo = NYLES_MG_XYZPERIO;
    else if (d->periodic_x && d->periodic_y) topo = NYLES_MG_XYPERIO;
    else if (d->periodic_x) topo = NYLES_MG_XPERIO;
    else if (d->periodic_y) topo = NYLES_MG_YPERIO;
    else topo = NYLES_MG_CLOSED;
    if (d->periodic_z && !(d->periodic_x && d->periodic_y)) {
        delete m;
        set_error("z-periodic geometry needs x and y periodic (perio_xyz)");
        return NYLES_UNSUPPORTED;
    }
    m->topo = topo;
    m->nstage = scheme == NYLES_SCHEME_RK3_SSP ? 3 : (scheme == NYLES_SCHEME_LFAM3 ? 2 : 1);
    rc = model_layout(m, 1, 0);
    if (rc) { delete m; return rc; }
    *out = m;
    return NYLES_OK;
}

int nyles_model_destroy(NylesModel* m) { delete m; return NYLES_OK; }

int nyles_model_workspace_bytes(const NylesModel* m, size_t* bytes) {
    if (!m || !bytes) { set_error("null argument"); return NYLES_BAD_ARG; }
    *bytes = m->bytes;
    return NYLES_OK;
}

int nyles_model_bind(NylesModel* m, void* const* fields, void* const* regs, void* workspace) {
    if (!m || !fields || !regs || !workspace) { set_error("null argument"); return NYLES_BAD_ARG; }
    if (((uintptr_t)workspace) & 255) { set_error("workspace must be 256-byte aligned"); return NYLES_BAD_ARG; }
    for (int i = 0; i < NYLES_F_T0 + m->d.n_tracers; ++i) {
        if (!fields[i]) { set_error("null field pointer"); return NYLES_BAD_ARG; }
        m->fields[i] = fields[i];
    }
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < m->nprog; ++q) {
            void* p = regs[r * m->nprog + q];
            if (!p) { set_error("null register pointer"); return NYLES_BAD_ARG; }
            m->regs[r][q] = p;
        }
    m->ws = (char*)workspace;
    m->mg.ws = m->ws + m->mg_off;
    m->bound = true;
    return mg_zero_scalars(&m->mg);
}

int nyles_model_set_mg_params(NylesModel* m, double tol, int maxite, double omega) {
    if (!m || maxite < 0 || !(tol >= 0.0) || !(omega > 0.0)) { set_error("bad multigrid parameters"); return NYLES_BAD_ARG; }
    m->mg.tol = tol; m->mg.maxite = maxite; m->mg.omega = omega;
    return NYLES_OK;
}

int nyles_model_set_mg_krylov(NylesModel* m, int on) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    if (m->gexec) { set_error("release the captured graph before changing the solver"); return NYLES_BAD_ARG; }
    return set_krylov(&m->mg, on);
}

int nyles_model_set_mg_warm_start(NylesModel* m, int mode) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    if (mode < 0 || mode > 4) { set_error("warm start mode must be 0..4"); return NYLES_BAD_ARG; }
    if (m->gexec) { set_error("release the captured graph before changing the warm start"); return NYLES_BAD_ARG; }
    if (mode && m->precision != NYLES_MIXED) {
        set_error("per-stage warm starts are provided for the mixed-precision solve only (the FP64 solve keeps "
                  "the reference's warm start)");
        return NYLES_UNSUPPORTED;
    }
    const int nsol = mode ? m->nstage : 1, nhist = mode >= 2 ? mode - 1 : 0;
    if (!m->bound) {   // size the workspace for this warm start
        int rc = model_layout(m, nsol, nhist);
        if (rc) return rc;
    } else if (nsol > m->mg.nsol || nhist > m->mg.nhist) {
        set_error("the bound workspace holds the arrays of a smaller warm start: select this one before "
                  "nyles_model_workspace_bytes and nyles_model_bind");
        return NYLES_BAD_ARG;
    }
    m->warm_per_stage = mode ? 1 : 0;
    m->mg.extrap = nhist;
    m->mg.cur_sol = 0;
    return mg_reset_history(&m->mg);
}

int nyles_model_reset_scheme(NylesModel* m) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    m->lf_first = true;
    return NYLES_OK;
}

int nyles_model_get_first_step(const NylesModel* m, int* pending) {
    if (!m || !pending) { set_error("null argument"); return NYLES_BAD_ARG; }
    *pending = m->lf_first ? 1 : 0;
    return NYLES_OK;
}

int nyles_model_set_first_step(NylesModel* m, int pending) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    m->lf_first = pending != 0;
    return NYLES_OK;
}

int nyles_model_mg_stats(const NylesModel* m, NylesMgStats* stats) {
    if (!m || !stats) { set_error("null argument"); return NYLES_BAD_ARG; }
    *stats = m->mg.stats;
    if (m->graph_launches > 0) {   // solves run inside graphs keep their statistics on the device
        NylesModel* mm = const_cast<NylesModel*>(m);
        MgDeviceStats ds;
        int rc = mg_read_device_stats(&mm->mg, mm->last_stream, &ds);
        if (rc) return rc;
        const long long vc = ds.vcycles;
        if (vc > mm->vcycles_counted) {
            note_launch((int)((vc - mm->vcycles_counted) * mm->graph_body_kernels));
            mm->vcycles_counted = vc;
        }
        if (m->last_solve_graph) {
            stats->nite = ds.nite;
            stats->res = ds.res;
        }
        stats->vcycles += vc;
        stats->solves += m->graph_launches * m->graph_solves;
        stats->not_converged += (int)ds.not_converged;
        stats->nonfinite += (int)ds.nonfinite;
    }
    return NYLES_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ orchestration
namespace nyles {

template <typename T>
static int model_rhs(NylesModel* m, int reg, int last, double t, cudaStream_t st, bool interior = false) {
    StencilPtrs<T> s = field_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->fields));
    ProgPtrs<T> ds = prog_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->regs[reg]));
    // Euler3d projects before its halo fill (core/model_les_euler.py:96-125): the
    // divergence next to the halo reads updated halo velocities, so their tendencies count
    if (m->d.model == NYLES_MODEL_EULER3D) interior = false;
    ProfScope ps(&m->prof, 0, st);
    int rc = launch_rhs<T>(&m->d, m->g, s, ds, rhs_terms(&m->d, last), st, interior, m->bat);
    // user forcing, core/model_les.py:143-144: called with the stage's register set and
    // time; it enqueues its own work on `st`
    if (!rc && m->forcing) m->forcing(m->forcing_user, reg, t, (void*)st);
    return rc;
}

// compute_p (core/projection.py:39-87): divergence of U = u/dx^2 into the multigrid
// right-hand side (and div), solve, p = x*dx^2, u -= grad p; then fill u
template <typename T>
static int model_pressure_projection(NylesModel* m, cudaStream_t st) {
    StencilPtrs<T> s = field_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->fields));
    int rc;
    T* uf[3] = {s.f[NYLES_F_U_I], s.f[NYLES_F_U_J], s.f[NYLES_F_U_K]};
    void* mgb = mg_level_ptr(&m->mg, 1, 2);
    void* mgx = mg_level_ptr(&m->mg, 1, 1);
    {
        ProfScope ps(&m->prof, 3, st);
        if constexpr (sizeof(T) == sizeof(double))
            rc = launch_div<T, double>(&m->d, m->g, s, reinterpret_cast<double*>(mgb), st);
        else
            rc = launch_div_df(&m->d, m->g, field_ptrs<float>(&m->d, reinterpret_cast<float* const*>(m->fields)),
                               reinterpret_cast<float2*>(mgb), st, m->bat);
        if (rc) return rc;
    }
    {
        ProfScope ps(&m->prof, 4, st);
        m->mg.prof = m->prof.on ? &m->prof : nullptr;
        if (m->gb) {
            if ((rc = mg_solve_graph(&m->mg, *m->gb))) return rc;
            ++m->graph_solves;
        } else {
            if ((rc = mg_solve(&m->mg, st))) return rc;
            m->last_solve_graph = false;
        }
    }
    {
        ProfScope ps(&m->prof, 5, st);
        if constexpr (sizeof(T) == sizeof(double))
            rc = launch_correct<T, double>(&m->d, m->g, s, reinterpret_cast<const double*>(mgx), m->d.dx2, st);
        else
            rc = launch_correct_df(m->g, field_ptrs<float>(&m->d, reinterpret_cast<float* const*>(m->fields)),
                                   reinterpret_cast<const float2*>(mgx), m->d.dx2, st, m->bat);
        if (rc) return rc;
    }
    ProfScope ps(&m->prof, 2, st);
    return launch_fill<T>(m->g, uf, 3, st, m->bat);
}

// core/model_les.py:98-127 ; core/model_les_euler.py:96-125 ; the advection model fills
// b only (core/model_advection.py:33-35)
// `stage`: index of the projection within the time step (selects the per-stage warm
// start of a mixed-precision model that keeps them)
template <typename T>
static int model_diagnose(NylesModel* m, cudaStream_t st, int stage = 0) {
    m->mg.cur_sol = (m->warm_per_stage && stage < m->mg.nsol) ? stage : 0;
    StencilPtrs<T> s = field_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->fields));
    int rc;
    T* uf[4] = {s.f[NYLES_F_B], s.f[NYLES_F_U_I], s.f[NYLES_F_U_J], s.f[NYLES_F_U_K]};
    if (m->d.model == NYLES_MODEL_ADVECTION) {
        ProfScope ps(&m->prof, 2, st);
        return launch_fill<T>(m->g, uf, 1, st);
    }
    if (m->d.model != NYLES_MODEL_EULER3D) {
        ProfScope ps(&m->prof, 2, st);
        if ((rc = launch_fill<T>(m->g, uf, 4, st, m->bat))) return rc;
    }
    if ((rc = model_pressure_projection<T>(m, st))) return rc;
    ProfScope ps(&m->prof, 6, st);
    return launch_diag<T>(&m->d, m->g, s, m->d.model != NYLES_MODEL_LINEAR, st, m->bat);
}

// Advection.make_u_divergentfree (core/model_advection.py:38-53) with the projection of
// diagnose_var: fill u, project, U = u/dx^2, div of U (evaluated at the periodic
// image, i.e. with its halo filled)
template <typename T>
static int model_project(NylesModel* m, cudaStream_t st) {
    StencilPtrs<T> s = field_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->fields));
    int rc;
    T* uf[3] = {s.f[NYLES_F_U_I], s.f[NYLES_F_U_J], s.f[NYLES_F_U_K]};
    if ((rc = launch_fill<T>(m->g, uf, 3, st))) return rc;
    if ((rc = model_pressure_projection<T>(m, st))) return rc;
    if ((rc = launch_diag<T>(&m->d, m->g, s, 0, st))) return rc;
    void* mgb = mg_level_ptr(&m->mg, 1, 2);   // overwritten: the right-hand side is scratch
    if constexpr (sizeof(T) == sizeof(double))
        return launch_div<T, double>(&m->d, m->g, s, reinterpret_cast<double*>(mgb), st);
    else
        return launch_div_df(&m->d, m->g, field_ptrs<float>(&m->d, reinterpret_cast<float* const*>(m->fields)),
                             reinterpret_cast<float2*>(mgb), st);
}

template <typename T>
static int model_update(NylesModel* m, int kind, int ra, int rb, int rc_, double dt, cudaStream_t st) {
    StencilPtrs<T> s = field_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->fields));
    ProgPtrs<T> sp = state_prog<T>(&m->d, s);
    auto reg = [&](int r) { return prog_ptrs<T>(&m->d, r >= 0 ? reinterpret_cast<T* const*>(m->regs[r]) : nullptr); };
    ProfScope ps(&m->prof, 1, st);
    return launch_update<T>(m->g, m->nprog, sp, reg(ra), reg(rb), reg(rc_), kind, dt, st, m->bat);
}

// core/timescheme.py:113-221
template <typename T>
static int model_forward(NylesModel* m, double t, double dt, cudaStream_t st) {
    int rc;
    if (m->scheme == NYLES_SCHEME_RK3_SSP) {
        if ((rc = model_rhs<T>(m, 0, 0, t, st, true))) return rc;
        if ((rc = model_update<T>(m, UPD_EULER, 0, -1, -1, dt, st))) return rc;
        if ((rc = model_diagnose<T>(m, st, 0))) return rc;
        if ((rc = model_rhs<T>(m, 1, 0, t + dt, st, true))) return rc;
        if ((rc = model_update<T>(m, UPD_RK3_2, 0, 1, -1, dt, st))) return rc;
        if ((rc = model_diagnose<T>(m, st, 1))) return rc;
        if ((rc = model_rhs<T>(m, 2, 1, t + dt * 0.5, st, true))) return rc;
        if ((rc = model_update<T>(m, UPD_RK3_3, 0, 1, 2, dt, st))) return rc;
        return model_diagnose<T>(m, st, 2);
    }
    if (m->scheme == NYLES_SCHEME_EF) {
        if ((rc = model_rhs<T>(m, 0, 1, t, st, true))) return rc;
        if ((rc = model_update<T>(m, UPD_EULER, 0, -1, -1, dt, st))) return rc;
        return model_diagnose<T>(m, st);
    }
    // LFAM3: registers 0 = dstate, 1 = stateb, 2 = state (n)
    if ((rc = model_rhs<T>(m, 0, 0, t, st, true))) return rc;
    if (m->lf_first) {
        if ((rc = model_update<T>(m, UPD_LF_FIRST, 0, 1, 2, dt, st))) return rc;
        m->lf_first = false;
        return model_diagnose<T>(m, st);
    }
    if ((rc = model_update<T>(m, UPD_LF_PRED, 0, 1, 2, dt, st))) return rc;
    if ((rc = model_diagnose<T>(m, st, 0))) return rc;
    if ((rc = model_rhs<T>(m, 0, 1, t + dt * 0.5, st, true))) return rc;
    if ((rc = model_update<T>(m, UPD_LF_CORR, 0, 1, 2, dt, st))) return rc;
    return model_diagnose<T>(m, st, 1);
}

}  // namespace nyles

extern "C" {

int nyles_model_forward(NylesModel* m, double t, double dt, void* stream) {
    if (!m || !m->bound) { set_error("model not bound"); return NYLES_BAD_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    return m->precision == NYLES_FP64 ? model_forward<double>(m, t, dt, st) : model_forward<float>(m, t, dt, st);
}

int nyles_model_diagnose(NylesModel* m, void* stream) {
    if (!m || !m->bound) { set_error("model not bound"); return NYLES_BAD_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    return m->precision == NYLES_FP64 ? model_diagnose<double>(m, st) : model_diagnose<float>(m, st);
}

int nyles_model_project(NylesModel* m, void* stream) {
    if (!m || !m->bound) { set_error("model not bound"); return NYLES_BAD_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    return m->precision == NYLES_FP64 ? model_project<double>(m, st) : model_project<float>(m, st);
}

int nyles_model_rhs(NylesModel* m, int reg, double t, int last, void* stream) {
    if (!m || !m->bound || reg < 0 || reg > 2) { set_error("model not bound or bad register"); return NYLES_BAD_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    return m->precision == NYLES_FP64 ? model_rhs<double>(m, reg, last, t, st) : model_rhs<float>(m, reg, last, t, st);
}

int nyles_model_set_forcing(NylesModel* m, nyles_forcing_fn fn, void* user) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    if (fn && m->gexec) { set_error("release the captured graph before attaching a forcing"); return NYLES_BAD_ARG; }
    m->forcing = fn;
    m->forcing_user = user;
    return NYLES_OK;
}

int nyles_model_max_U2(NylesModel* m, double* out, void* stream) {
    if (!m || !m->bound || !out) { set_error("model not bound or null output"); return NYLES_BAD_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    double* part = reinterpret_cast<double*>(m->ws + m->off_partial);
    double* dev = reinterpret_cast<double*>(m->ws + m->off_scalar);
    int rc;
    ProfScope ps(&m->prof, 7, st);
    if (m->precision == NYLES_FP64)
        rc = launch_max_U2<double>(m->g, field_ptrs<double>(&m->d, reinterpret_cast<double* const*>(m->fields)), part,
                                   m->npartial, dev, st);
    else
        rc = launch_max_U2<float>(m->g, field_ptrs<float>(&m->d, reinterpret_cast<float* const*>(m->fields)), part,
                                  m->npartial, dev, st);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(out, dev, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    rc = cuda_status(e, "max_U2 read-back");
    if (rc) return rc;
    if (!(*out == *out) || *out > 1.7976931348623157e308) { set_error("non-finite velocity"); return NYLES_BLOWUP; }
    return NYLES_OK;
}

extern "C++" {
template <typename T>
static int model_vfwork(NylesModel* m, const VfBox& box, double* out, cudaStream_t st) {
    StencilPtrs<T> s = field_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->fields));
    ProgPtrs<T> ds = prog_ptrs<T>(&m->d, reinterpret_cast<T* const*>(m->regs[0]));
    for (int c = 1; c <= 3; ++c) {
        cudaError_t e = cudaMemsetAsync(ds.p[c], 0, (size_t)m->g.vol * sizeof(T), st);
        if (e != cudaSuccess) return cuda_status(e, "vfwork register reset");
    }
    int rc = launch_rhs<T>(&m->d, m->g, s, ds, TERM_VF | TERM_ACCUMULATE, st);
    if (rc) return rc;
    double* part = reinterpret_cast<double*>(m->ws + m->off_partial);
    double* dev = reinterpret_cast<double*>(m->ws + m->off_scalar);
    return launch_vfwork<T>(m->g, s, ds, box, part, m->npartial, dev, st);
}
}  // extern "C++"

int nyles_model_vfwork(NylesModel* m, const long long* box, double* worksum, void* stream) {
    if (!m || !m->bound || !box || !worksum) { set_error("model not bound or null argument"); return NYLES_BAD_ARG; }
    VfBox b;
    for (int d = 0; d < 3; ++d) {
        const long long lo = box[2 * d], hi = box[2 * d + 1];
        if (lo < 0 || hi < lo || hi > m->g.N[d]) { set_error("vfwork: box outside the arrays"); return NYLES_BAD_ARG; }
        b.lo[d] = (int)lo;
        b.hi[d] = (int)hi;
    }
    cudaStream_t st = (cudaStream_t)stream;
    double* dev = reinterpret_cast<double*>(m->ws + m->off_scalar);
    int rc = m->precision == NYLES_FP64 ? model_vfwork<double>(m, b, worksum, st) : model_vfwork<float>(m, b, worksum, st);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(worksum, dev, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e, "vfwork read-back");
}

int nyles_model_profile(NylesModel* m, int enable) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    if (!enable) m->prof.flush();
    m->prof.on = enable != 0;
    return NYLES_OK;
}

int nyles_model_profile_read(NylesModel* m, double* ms, long long* count, int nphase) {
    if (!m || !ms || !count || nphase < 0) { set_error("bad argument"); return NYLES_BAD_ARG; }
    m->prof.flush();
    for (int i = 0; i < nphase && i < NYLES_NPHASE; ++i) {
        ms[i] = m->prof.ms[i];
        count[i] = m->prof.cnt[i];
        m->prof.ms[i] = 0.0;
        m->prof.cnt[i] = 0;
    }
    return NYLES_OK;
}

long long nyles_launch_count(void) { return g_launches.load(); }

}  // extern "C"

// Record nsteps steps of m (nsteps = 0: one diagnose_var) into a new graph (multigrid
// stop tests on the device); the kernels outside the multigrid loops and those of one
// loop iteration are counted.
static int record_steps(NylesModel* m, double dt, int nsteps, cudaGraph_t* graph, cudaGraphExec_t* exec,
                        long long* kernels, long long* body_kernels) {
    if (nsteps > 0 && m->scheme == NYLES_SCHEME_LFAM3 && m->lf_first) {
        set_error("LFAM3: run the first (Euler) step before capturing the steady step");
        return NYLES_BAD_ARG;
    }
    if (m->forcing) {
        set_error("a model with a user forcing cannot be captured (the forcing runs on the host)");
        return NYLES_BAD_ARG;
    }
    cudaError_t e;
    if (!m->cap_stream) {
        e = cudaStreamCreateWithFlags(&m->cap_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_status(e, "capture stream");
    }
    e = cudaGraphCreate(graph, 0);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphCreate");
    GraphBuilder gb;
    gb.graph = *graph;
    gb.st = m->cap_stream;
    const bool prof_on = m->prof.on;
    m->prof.on = false;   // event records are not allowed inside loop bodies
    m->gb = &gb;
    m->graph_solves = 0;
    const long long l0 = g_launches.load();
    gb.begin_segment();
    int rc = NYLES_OK;
    for (int s = 0; s < nsteps && !rc && !gb.error; ++s)
        rc = m->precision == NYLES_FP64 ? model_forward<double>(m, 0.0, dt, gb.st)
                                        : model_forward<float>(m, 0.0, dt, gb.st);
    if (nsteps == 0)
        rc = m->precision == NYLES_FP64 ? model_diagnose<double>(m, gb.st) : model_diagnose<float>(m, gb.st);
    gb.end_segment();
    m->gb = nullptr;
    m->prof.on = prof_on;
    const long long captured = g_launches.load() - l0;
    g_launches.fetch_sub(captured);   // nothing ran yet: launches are counted at replay
    if (!rc) rc = gb.error;
    if (!rc) {
        *body_kernels = gb.body_kernels;
        *kernels = captured - (long long)m->graph_solves * gb.body_kernels;
        e = cudaGraphInstantiate(exec, *graph, 0);
        if (e != cudaSuccess) rc = cuda_status(e, "cudaGraphInstantiate");
    }
    if (rc) {
        if (*graph) cudaGraphDestroy(*graph);
        *graph = nullptr;
        *exec = nullptr;
    }
    return rc;
}

extern "C" {

int nyles_model_capture(NylesModel* m, double dt, int nsteps) {
    if (!m || !m->bound || nsteps < 1) { set_error("model not bound or nsteps < 1"); return NYLES_BAD_ARG; }
    m->release_graph();
    return record_steps(m, dt, nsteps, &m->graph, &m->gexec, &m->graph_kernels, &m->graph_body_kernels);
}

int nyles_model_batch_capture(NylesModel* m, double dt, int nsteps, int nrun, NylesBatchTable* table,
                              NylesBatchGraph** out) {
    if (!m || !m->bound || nsteps < 0 || !out) { set_error("model not bound, nsteps < 0 or null output"); return NYLES_BAD_ARG; }
    *out = nullptr;
    if (nrun < 1 || nrun > NYLES_MAX_BATCH || !table || (((uintptr_t)table) & 7)) {
        set_error("batched capture: 1 <= nrun <= NYLES_BATCH_RUNS and an 8-byte aligned device table required");
        return NYLES_BAD_ARG;
    }
    const NylesDesc& d = m->d;
    if (m->precision != NYLES_MIXED || m->mg.krylov || d.model != NYLES_MODEL_LES || d.n_tracers != 0 ||
        d.tracer_diffusion != 0 || d.tracer_order != 0 || d.vf_order != 0) {
        set_error("batched steps cover the mixed-precision LES model with the stationary pressure solve, "
                  "no tracers and the reference's schemes");
        return NYLES_UNSUPPORTED;
    }
    NylesBatchGraph* g = new (std::nothrow) NylesBatchGraph;
    if (!g) { set_error("out of host memory"); return NYLES_CUDA_ERROR; }
    m->bat.tab = reinterpret_cast<BatchTab*>(table);
    m->bat.nrun = nrun;
    m->bat.gate = GATE_ACTIVE;
    m->mg.bat = m->bat;
    const int solves = m->graph_solves;   // of the one-run graph, if any
    int rc = record_steps(m, dt, nsteps, &g->graph, &g->exec, &g->kernels, &g->body_kernels);
    m->graph_solves = solves;
    m->bat = Bat();
    m->mg.bat = Bat();
    if (rc) { delete g; return rc; }
    *out = g;
    return NYLES_OK;
}

int nyles_batch_launch(NylesBatchGraph* g, void* stream) {
    if (!g || !g->exec) { set_error("no batched graph"); return NYLES_BAD_ARG; }
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphLaunch");
    note_launch((int)g->kernels);
    return NYLES_OK;
}

int nyles_batch_note_iterations(const NylesBatchGraph* g, long long iterations) {
    if (!g || iterations < 0) { set_error("null graph or negative count"); return NYLES_BAD_ARG; }
    note_launch((int)(iterations * g->body_kernels));
    return NYLES_OK;
}

int nyles_batch_destroy(NylesBatchGraph* g) {
    delete g;
    return NYLES_OK;
}

int nyles_model_device_stats(NylesModel* m, NylesMgStats* stats, void* stream) {
    if (!m || !m->bound || !stats) { set_error("model not bound or null output"); return NYLES_BAD_ARG; }
    MgDeviceStats ds;
    int rc = mg_read_device_stats(&m->mg, (cudaStream_t)stream, &ds);
    if (rc) return rc;
    *stats = NylesMgStats{};
    stats->nite = ds.nite;
    stats->res = ds.res;
    stats->vcycles = ds.vcycles;
    stats->not_converged = (int)ds.not_converged;
    stats->nonfinite = (int)ds.nonfinite;
    return NYLES_OK;
}

int nyles_model_graph_launch(NylesModel* m, void* stream) {
    if (!m || !m->gexec) { set_error("no captured graph"); return NYLES_BAD_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaGraphLaunch(m->gexec, st);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphLaunch");
    note_launch((int)m->graph_kernels);
    m->graph_launches += 1;
    m->last_solve_graph = true;
    m->last_stream = st;
    return NYLES_OK;
}

int nyles_model_graph_release(NylesModel* m) {
    if (!m) { set_error("null model"); return NYLES_BAD_ARG; }
    m->release_graph();
    return NYLES_OK;
}

}  // extern "C"
