// Geometric multigrid of the pressure projection, one rank (core/mgfor).
//
// Level arrays hold interior cells only. The ghost layers of the reference are implied:
// across a closed wall a ghost holds 0 and is "dry" (mask 0), in a periodic direction
// it is the periodic image of the interior (mod_halo.f90:235-262). With that, every
// operator coefficient of mgfor's setup (operators.f90:299-505) is a function of the
// cell position and is evaluated in the kernels instead of being stored:
//   diag  = number of wet face neighbours, idiag = 1/diag     (compute_diag)
//   Rcoef = 1/2 on every coarse interior cell                   (compute_Rcoef)
//   Pcoef = 1/(Wx*Wy*Wz), W = 3 + [coarse neighbour is wet]     (compute_Pcoef)
// The smoother's intermediate `y` on the ghost ring (basicoperators.f90:380-388) is 0
// across closed walls (its idiag and x are 0 there) and the periodic image otherwise.
//
// Kernel layout: blocks of 32 x 8 threads over (x, y); each thread marches over a chunk
// of z, keeping the z-1, z, z+1 values in registers. A block whose cells and stencil
// neighbours all lie inside the level takes a fast path with direct strided loads;
// only blocks touching the level's faces go through the ghost logic.
#include "nyles_internal.h"
#include <cstdlib>
#include <vector>
#include <cstring>

namespace nyles {

struct MgGeom {
    int n[3];          // interior extents z, y, x
    int per[3];
    double idiag[8];   // omega/diag for diag = 0..6 (0 -> 0): the damped inverse diagonal, host-computed
    double pcoef[8];   // 1/(Wx*Wy*Wz) indexed by the three "neighbour is wet" bits
    float fidiag[8];   // the same tables rounded to float: single-precision kernels read
    float fpcoef[8];   // these instead of converting (FP64 conversions use the FP64 pipe)
};
template <typename T> __device__ __forceinline__ T mg_idiag(const MgGeom& g, int k);
template <> __device__ __forceinline__ double mg_idiag<double>(const MgGeom& g, int k) { return g.idiag[k]; }
template <> __device__ __forceinline__ float mg_idiag<float>(const MgGeom& g, int k) { return g.fidiag[k]; }
template <typename T> __device__ __forceinline__ T mg_pcoef(const MgGeom& g, int k);
template <> __device__ __forceinline__ double mg_pcoef<double>(const MgGeom& g, int k) { return g.pcoef[k]; }
template <> __device__ __forceinline__ float mg_pcoef<float>(const MgGeom& g, int k) { return g.fpcoef[k]; }

// Scalars of the solve in the workspace: [0] last sum(r^2), [1] sum(b^2), [2] res,
// [3] nite of the current solve, [4] V-cycles since creation, [5] and [6] the scale of
// the mixed-precision residual sums and its inverse square.
// device scalars of the solver (SC_COUNT <= 16 doubles, zeroed when the workspace is
// bound): slots 7-12 belong to the Krylov solve; SC_NCONV counts graph-mode solves
// that stopped at maxite above tol, SC_NONFINITE graph-mode solves stopped by a
// non-finite norm
enum { SC_RR = 0, SC_NORMB = 1, SC_RES = 2, SC_NITE = 3, SC_TOTAL = 4, SC_SCALE = 5, SC_INVSCALE2 = 6,
       SC_ZQ = 7, SC_PQ = 8, SC_PR = 9, SC_BETA = 10, SC_ALPHA = 11, SC_ZMEAN = 12,
       SC_NCONV = 13, SC_NONFINITE = 14, SC_COUNT = 15 };
static_assert(SC_COUNT <= 16, "multigrid scalars exceed their 16-double slot");

constexpr int MG_BX = 32, MG_BY = 8, MG_ZC = 8;    // stencil kernels
constexpr int MG_RZC = 2;                          // restriction (coarse z per thread)
constexpr int MG_DFZC = 8;                         // float-pair residual

__device__ __forceinline__ long long mg_at(const MgGeom& g, int z, int y, int x) {
    return ((long long)z * g.n[1] + y) * g.n[2] + x;
}

// Value at (z, y, x), one cell outside the interior at most: periodic image, or 0
// across a closed wall. Branch-free on purpose: the index is folded into range, the
// load always reads an interior cell and the wall case is a select. With early
// returns before the load, the fused residual-restriction kernel built by ptxas -O3
// (CUDA 13.0, sm_103a) returned wrong sums next to closed x walls, while the same
// source was exact on the host and with -Xptxas -O0; this form is exact in both.
template <typename T>
__device__ __forceinline__ T mg_rd(const T* __restrict__ a, const MgGeom& g, int z, int y, int x) {
    bool ok = true;
    int q[3] = {z, y, x};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int n = g.n[k];
        const bool lo = q[k] < 0, hi = q[k] >= n;
        ok = ok && (g.per[k] || !(lo || hi));
        q[k] = lo ? q[k] + n : (hi ? q[k] - n : q[k]);
        q[k] = min(max(q[k], 0), n - 1);
    }
    const T v = a[((long long)q[0] * g.n[1] + q[1]) * g.n[2] + q[2]];
    return ok ? v : T(0);
}

__device__ __forceinline__ int mg_diag(const MgGeom& g, int z, int y, int x) {
    int d = 0;
    d += g.per[0] ? 2 : ((z > 0) + (z < g.n[0] - 1));
    d += g.per[1] ? 2 : ((y > 0) + (y < g.n[1] - 1));
    d += g.per[2] ? 2 : ((x > 0) + (x < g.n[2] - 1));
    return d;
}

// sum of the six face neighbours in mgfor's order: x-1, x+1, y-1, y+1, z-1, z+1
template <typename T>
__device__ __forceinline__ T mg_nsum(const T* __restrict__ a, const MgGeom& g, int z, int y, int x) {
    return ((((mg_rd(a, g, z, y, x - 1) + mg_rd(a, g, z, y, x + 1)) + mg_rd(a, g, z, y - 1, x)) +
             mg_rd(a, g, z, y + 1, x)) + mg_rd(a, g, z - 1, y, x)) + mg_rd(a, g, z + 1, y, x);
}

// residual r = msk*(b + diag*x - sum(x_nb)) (basicoperators.f90:300-323), ghost logic
template <typename T>
__device__ __forceinline__ T mg_resid(const T* __restrict__ x, const T* __restrict__ b, const MgGeom& g, int z, int y,
                                      int xx) {
    const long long c = mg_at(g, z, y, xx);
    const T dg = T(mg_diag(g, z, y, xx));
    return (b[c] + dg * x[c]) - mg_nsum(x, g, z, y, xx);
}
// same with every neighbour inside the level (diag = 6), direct loads
template <typename T>
__device__ __forceinline__ T mg_resid_in(const T* __restrict__ x, const T* __restrict__ b, long long c, long long sy,
                                         long long sz) {
    return (b[c] + T(6) * x[c]) - (((((x[c - 1] + x[c + 1]) + x[c - sy]) + x[c + sy]) + x[c - sz]) + x[c + sz]);
}

// ---- per-cell operators with the ghost logic (used at level faces and on the levels
// held in shared memory by k_mg_bottom)
// damped Jacobi value at (z, y, x): (1-omega)*in + omega*(sum(in_nb) - b)*idiag
template <typename T>
__device__ __forceinline__ T mg_jacobi_cell(const MgGeom& g, const T* __restrict__ in, const T* __restrict__ b, int z,
                                            int y, int x, T cff1, T omega) {
    const long long c = mg_at(g, z, y, x);
    const T idg = mg_idiag<T>(g, mg_diag(g, z, y, x));
    (void)omega;
    return cff1 * in[c] + (mg_nsum(in, g, z, y, x) - b[c]) * idg;
}
// sum of the residuals of the 8 children of coarse cell (z, y, x)
template <typename T>
__device__ __forceinline__ T mg_restrict_cell(const MgGeom& gf, const T* __restrict__ xf, const T* __restrict__ bf,
                                              int z, int y, int x) {
    const int i = 2 * x, j = 2 * y, k = 2 * z;
    T s = mg_resid(xf, bf, gf, k, j, i);
    s = s + mg_resid(xf, bf, gf, k, j, i + 1);
    s = s + mg_resid(xf, bf, gf, k, j + 1, i);
    s = s + mg_resid(xf, bf, gf, k, j + 1, i + 1);
    s = s + mg_resid(xf, bf, gf, k + 1, j, i);
    s = s + mg_resid(xf, bf, gf, k + 1, j, i + 1);
    s = s + mg_resid(xf, bf, gf, k + 1, j + 1, i);
    s = s + mg_resid(xf, bf, gf, k + 1, j + 1, i + 1);
    return s;
}
// 9-3-3-1 prolongation increment of fine cell (z, y, x)
template <typename T>
__device__ __forceinline__ T mg_prolong_cell(const MgGeom& gf, const MgGeom& gc, const T* __restrict__ xc, int z,
                                             int y, int x) {
    const int ic = x >> 1, jc = y >> 1, kc = z >> 1;
    const int si = (x & 1) ? 1 : -1, sj = (y & 1) ? 1 : -1, sk = (z & 1) ? 1 : -1;
    auto plane = [&](int kk) -> T {
        return ((T(9) * mg_rd(xc, gc, kk, jc, ic) + T(3) * mg_rd(xc, gc, kk, jc, ic + si)) +
                T(3) * mg_rd(xc, gc, kk, jc + sj, ic)) + mg_rd(xc, gc, kk, jc + sj, ic + si);
    };
    const T bpl = plane(kc);
    const T opl = plane(kc + sk);
    auto wet = [&](int d, int v) -> int { return (gc.per[d] || (v >= 0 && v < gc.n[d])) ? 1 : 0; };
    const T pcoef = mg_pcoef<T>(gf, wet(2, ic + si) | (wet(1, jc + sj) << 1) | (wet(0, kc + sk) << 2));
    return pcoef * (T(3) * bpl + opl);
}

// ---- grid kernels: one thread per (x, y) column and chunk of z
// The neighbours of a thread's fixed coordinate along one direction: element offsets
// of the cells at c-1 and c+1 and whether they are wet. Outside the level a neighbour
// is the periodic image or, across a closed wall, dry: its offset is then 0 (the cell
// itself, a valid address) and the value read is replaced by 0 — loads are never
// skipped (see mg_rd).
struct MgNb {
    long long om, op;
    bool wm, wp;
};
__device__ __forceinline__ MgNb mg_nb(int c, int n, int per, long long stride) {
    MgNb r;
    r.wm = c > 0 || per;
    r.wp = c < n - 1 || per;
    r.om = c > 0 ? -stride : (per ? (long long)(n - 1) * stride : 0);
    r.op = c < n - 1 ? stride : (per ? -(long long)(n - 1) * stride : 0);
    return r;
}
template <typename T>
__device__ __forceinline__ T mg_ldw(const T* __restrict__ a, long long c, bool wet) {
    const T v = a[c];
    return wet ? v : T(0);
}

// per-block partial sum (one double per block, block index order); bz = the block's z
// index within its run's grid (blockIdx.z outside batched launches)
__device__ __forceinline__ void block_partial(double s, double* __restrict__ partial, int bz) {
    __shared__ double sm[MG_BX * MG_BY / 32];
    const int tid = threadIdx.y * MG_BX + threadIdx.x;
    s = warp_sum(s);
    if ((tid & 31) == 0) sm[tid >> 5] = s;
    __syncthreads();
    if (tid < 32) {
        double t = (tid < MG_BX * MG_BY / 32) ? sm[tid] : 0.0;
        t = warp_sum(t);
        if (tid == 0) partial[(bz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = t;
    }
}

// two per-block partial sums at once
__device__ __forceinline__ void block_partial2(double s, double t, double* __restrict__ ps,
                                               double* __restrict__ pt, int bz) {
    __shared__ double sm[2][MG_BX * MG_BY / 32];
    const int tid = threadIdx.y * MG_BX + threadIdx.x;
    s = warp_sum(s);
    t = warp_sum(t);
    if ((tid & 31) == 0) {
        sm[0][tid >> 5] = s;
        sm[1][tid >> 5] = t;
    }
    __syncthreads();
    if (tid < 32) {
        double a = (tid < MG_BX * MG_BY / 32) ? sm[0][tid] : 0.0;
        double b = (tid < MG_BX * MG_BY / 32) ? sm[1][tid] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        if (tid == 0) {
            const int blk = (bz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            ps[blk] = a;
            pt[blk] = b;
        }
    }
}

// FP32 forms of block_partial and block_partial2 for kernels whose per-thread sums are
// FP32: the warp and block stages add in float and only the block total is stored as a
// double (times `scale`). On GB300 the FP64 pipe is narrow: the double shuffles, adds
// and conversions of a 256-thread reduction took a visible share of a level-0 pass.
__device__ __forceinline__ void block_partial_f(float s, double scale, double* __restrict__ partial, int bz) {
    __shared__ float smf[MG_BX * MG_BY / 32];
    const int tid = threadIdx.y * MG_BX + threadIdx.x;
    s = warp_sum(s);
    if ((tid & 31) == 0) smf[tid >> 5] = s;
    __syncthreads();
    if (tid < 32) {
        float t = (tid < MG_BX * MG_BY / 32) ? smf[tid] : 0.f;
        t = warp_sum(t);
        if (tid == 0) partial[(bz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = (double)t * scale;
    }
}
__device__ __forceinline__ void block_partial2_f(float s, float t, double* __restrict__ ps, double* __restrict__ pt,
                                                 int bz) {
    __shared__ float smf[2][MG_BX * MG_BY / 32];
    const int tid = threadIdx.y * MG_BX + threadIdx.x;
    s = warp_sum(s);
    t = warp_sum(t);
    if ((tid & 31) == 0) {
        smf[0][tid >> 5] = s;
        smf[1][tid >> 5] = t;
    }
    __syncthreads();
    if (tid < 32) {
        float a = (tid < MG_BX * MG_BY / 32) ? smf[0][tid] : 0.f;
        float b = (tid < MG_BX * MG_BY / 32) ? smf[1][tid] : 0.f;
        a = warp_sum(a);
        b = warp_sum(b);
        if (tid == 0) {
            const int blk = (bz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            ps[blk] = (double)a;
            pt[blk] = (double)b;
        }
    }
}

// ---- the final sum of a reduction folded into the kernel that stores the partials
// The block that stores its partial last (a ticket from an atomic counter, taken after
// a fence that orders every block's partial store before its ticket) adds all partials
// in block order and finishes the reduction itself, instead of a separate one-block
// launch after the kernel; it resets the counter for the next launch. `ticket` lies in
// the solver's workspace (zeroed when the workspace is bound; batched launches: each
// run's own). The sum's order depends on the grid only, so results are deterministic.
struct MgFin {
    unsigned int* ticket = nullptr;   // null: the partials are summed by a later launch
    double* sc = nullptr;             // the solve's scalars (shifted to the run in batched launches)
    int k = 0;                        // Krylov iteration (-1: read sc[SC_NITE])
    double vol = 0.0;                 // level-0 cells
};
// Thread (0, 0) stored the block's partial (block_partial*): it alone fences that store
// before taking the ticket (a fence in every thread stalled every block on its way out).
__device__ __forceinline__ bool mg_last_block(unsigned int* ticket, unsigned int nblk) {
    __shared__ unsigned int s_last;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        s_last = (t == nblk - 1) ? 1u : 0u;
        if (s_last) atomicExch(ticket, 0u);
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}
// totals of n partials of one or two sums, added in a fixed order by the threads of a
// MG_BX x MG_BY block (loads through L2: other blocks of the launch stored them); the
// result is valid in thread (0, 0)
__device__ __forceinline__ double2 mg_block_total2(const double* pa, const double* pb, int n) {
    __shared__ double sm[2][MG_BX * MG_BY / 32];
    const int tid = threadIdx.y * MG_BX + threadIdx.x;
    double a = 0.0, b = 0.0;
    for (int i = tid; i < n; i += MG_BX * MG_BY) {
        a += __ldcg(pa + i);
        if (pb) b += __ldcg(pb + i);
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if ((tid & 31) == 0) {
        sm[0][tid >> 5] = a;
        sm[1][tid >> 5] = b;
    }
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (tid < 32) {
        double x = (tid < MG_BX * MG_BY / 32) ? sm[0][tid] : 0.0;
        double y = (tid < MG_BX * MG_BY / 32) ? sm[1][tid] : 0.0;
        x = warp_sum(x);
        y = warp_sum(y);
        r = make_double2(x, y);
    }
    return r;
}
// beta = -(z.q)/(p.q) of the previous iteration (0 on the first: k = iteration of this
// solve, or sc[SC_NITE] when k < 0) stored as a float, and the mean of z (float)
__device__ __forceinline__ void fcg_set_beta(double zq, double zs, double vol, double* sc, int k) {
    const int it = k >= 0 ? k : (int)sc[SC_NITE];
    const double pq = sc[SC_PQ];
    double beta = (it > 0 && pq != 0.0) ? -zq / pq : 0.0;
    if (!isfinite(beta)) beta = 0.0;
    double zmean = zs / vol;
    if (!isfinite(zmean)) zmean = 0.0;
    sc[SC_ZQ] = zq;
    reinterpret_cast<float*>(sc + SC_BETA)[0] = (float)beta;
    reinterpret_cast<float*>(sc + SC_ZMEAN)[0] = (float)zmean;
}
// alpha = (p.r)/(p.q) stored as a float pair
__device__ __forceinline__ void fcg_set_alpha(double pq, double pr, double* sc) {
    double alpha = pq != 0.0 ? pr / pq : 0.0;
    if (!isfinite(alpha)) alpha = 0.0;
    sc[SC_PQ] = pq;
    sc[SC_PR] = pr;
    const float hi = (float)alpha;
    float2* a2 = reinterpret_cast<float2*>(sc + SC_ALPHA);
    *a2 = make_float2(hi, (float)(alpha - (double)hi));
}

// one damped-Jacobi half-sweep, out = (1-omega)*in + omega*(sum(in_nb) - b)*idiag
// (basicoperators.f90:379-398). MODE 0 stores it; MODE 1 adds it to the float-pair
// solution `acc` instead (mixed precision: the correction of iterative refinement,
// fused into the last half-sweep of the V-cycle); MODE 2 stores it and sums out*dot
// and out per block into `partial` and `partial2` (the Krylov solve: z.q of the new
// preconditioned residual against the previous direction's image, and the sum of z).
// BAT: batched launch over the runs of `bat` (pointers shifted to each run's memory)
template <typename T, int MODE, bool BAT = false>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_jacobi(const MgGeom g, const T* __restrict__ in,
                                                            const T* __restrict__ b, T* __restrict__ out, T omega,
                                                            float2* __restrict__ acc, const T* __restrict__ dot,
                                                            double* __restrict__ partial,
                                                            double* __restrict__ partial2, const Bat bat = Bat()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        in = bshift(in, dlt);
        b = bshift(b, dlt);
        out = bshift(out, dlt);
        acc = bshift(acc, dlt);
        dot = bshift(dot, dlt);
        partial = bshift(partial, dlt);
        partial2 = bshift(partial2, dlt);
    }
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    float sdot = 0.f, ssum = 0.f;
    if (x < g.n[2] && y < g.n[1]) {
        const int nz = g.n[0], z0 = bz * MG_ZC;
        const long long sy = g.n[2], sz = (long long)g.n[1] * g.n[2];
        const MgNb nx = mg_nb(x, g.n[2], g.per[2], 1), ny = mg_nb(y, g.n[1], g.per[1], sy);
        const int dxy = (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp;
        const T cff1 = T(1) - omega;
        const long long c0 = mg_at(g, z0, y, x);
        // neighbour sum in mgfor's order x-1, x+1, y-1, y+1, z-1, z+1
        auto cell = [&](long long c, T zm, T x0, T zp, T idg) -> T {
            const T s = ((((mg_ldw(in, c + nx.om, nx.wm) + mg_ldw(in, c + nx.op, nx.wp)) +
                           mg_ldw(in, c + ny.om, ny.wm)) + mg_ldw(in, c + ny.op, ny.wp)) + zm) + zp;
            return cff1 * x0 + (s - b[c]) * idg;
        };
        // dv: the cell's value of `dot` (MODE 2)
        auto put = [&](long long c, T v, T dv) {
            if (MODE == 1) {
                acc[c] = df_add_f(acc[c], (float)v);
            } else {
                out[c] = v;
                if (MODE == 2) {
                    sdot = __fmaf_rn((float)v, (float)dv, sdot);
                    ssum = __fadd_rn(ssum, (float)v);
                }
            }
        };
        if (z0 + MG_ZC <= nz) {
            // full chunk: fixed trip count, fully unrolled, so that every load of the chunk
            // is issued before the first result is needed
            const MgNb lo = mg_nb(z0, nz, g.per[0], sz), hi = mg_nb(z0 + MG_ZC - 1, nz, g.per[0], sz);
            T col[MG_ZC + 2];
            col[0] = mg_ldw(in, c0 + lo.om, lo.wm);
#pragma unroll
            for (int k = 1; k <= MG_ZC; ++k) col[k] = in[c0 + (k - 1) * sz];
            col[MG_ZC + 1] = mg_ldw(in, c0 + (MG_ZC - 1) * sz + hi.op, hi.wp);
            const T idg = mg_idiag<T>(g, dxy + 2);
            const T idg_lo = mg_idiag<T>(g, dxy + 1 + (int)lo.wm);
            const T idg_hi = mg_idiag<T>(g, dxy + 1 + (int)hi.wp);
#pragma unroll
            for (int k = 0; k < MG_ZC; ++k) {
                const long long c = c0 + k * sz;
                put(c, cell(c, col[k], col[k + 1], col[k + 2], k == 0 ? idg_lo : (k == MG_ZC - 1 ? idg_hi : idg)),
                    (MODE == 2) ? dot[c] : T(0));
            }
        } else {
            for (int z = z0; z < nz; ++z) {   // last, partial chunk
                const long long c = mg_at(g, z, y, x);
                const MgNb nzb = mg_nb(z, nz, g.per[0], sz);
                const T idg = mg_idiag<T>(g, dxy + (int)nzb.wm + (int)nzb.wp);
                put(c, cell(c, mg_ldw(in, c + nzb.om, nzb.wm), in[c], mg_ldw(in, c + nzb.op, nzb.wp), idg),
                    (MODE == 2) ? dot[c] : T(0));
            }
        }
    }
    if constexpr (MODE == 2) {
        if constexpr (sizeof(T) == sizeof(float))
            block_partial2_f(sdot, ssum, partial, partial2, bz);
        else
            block_partial2((double)sdot, (double)ssum, partial, partial2, bz);
    }
}

// k_mg_jacobi for float levels with 4 consecutive x cells per thread (16-byte accesses;
// the x neighbours of a vector from the adjacent lanes, loaded at the warp's ends and at
// the level's x faces) and z-chunks of V4_ZC cells; needs nx and nz divisible by 4 and
// V4_ZC. Same per-cell arithmetic and modes as k_mg_jacobi.
constexpr int V4_ZC = 4;

// value at c, or 0 across a closed wall (mg_ldw for the float vector kernels)
__device__ __forceinline__ float mg_ldw_f(const float* __restrict__ a, long long c, bool wet) {
    const float v = a[c];
    return wet ? v : 0.f;
}

// One block of the vector half-sweep: block (bx, by, bz) of the grid grid_v4(n, ZC);
// MODE 2 accumulates the block's sums of out*dot and out into sdot and ssum.
template <int MODE, int ZC>
__device__ __forceinline__ void mg_jacobi_v4_blk(const MgGeom& g, const float* __restrict__ in,
                                                 const float* __restrict__ b, float* __restrict__ out, float omega,
                                                 float2* __restrict__ acc, const float* __restrict__ dot, int bx,
                                                 int by, int bz, float& sdot, float& ssum) {
    const int nx = g.n[2], ny = g.n[1], nz = g.n[0];
    const int nx4 = nx >> 2;
    const int lane = threadIdx.x;
    const int xv = bx * MG_BX + lane;
    const int y = by * MG_BY + threadIdx.y;
    // idle lanes shadow the last vector of the row (every lane takes part in the
    // shuffles); only active lanes store and sum
    const bool act = xv < nx4 && y < ny;
    const int x0 = min(xv, nx4 - 1) * 4, ys = min(y, ny - 1);
    const long long sy = nx, sz = (long long)ny * nx;
    const MgNb nyb = mg_nb(ys, ny, g.per[1], sy);
    const bool wl = x0 > 0 || g.per[2], wr = x0 + 4 < nx || g.per[2];
    const long long ol = x0 > 0 ? -1 : (g.per[2] ? (long long)(nx - 1) : 0);
    const long long orr = x0 + 4 < nx ? 4 : (g.per[2] ? (long long)(4 - nx) : 0);
    const bool ownl = lane == 0 || x0 == 0, ownr = lane == MG_BX - 1 || x0 + 4 >= nx;
    int dgx[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int xx = x0 + e;
        dgx[e] = (int)(xx > 0 || g.per[2]) + (int)(xx < nx - 1 || g.per[2]) + (int)nyb.wm + (int)nyb.wp;
    }
    const float cff1 = 1.f - omega;
    const int zb = bz * ZC;
    const long long c00 = (long long)ys * sy + x0;
    auto ld4 = [&](const float* a, long long c) { return *reinterpret_cast<const float4*>(a + c); };
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    auto zrow = [&](int zz) -> float4 {
        if (zz < 0) return g.per[0] ? ld4(in, c00 + (long long)(nz - 1) * sz) : zero4;
        if (zz >= nz) return g.per[0] ? ld4(in, c00) : zero4;
        return ld4(in, c00 + (long long)zz * sz);
    };
    float4 zm = zrow(zb - 1), zc = zrow(zb);
#pragma unroll
    for (int k = 0; k < ZC; ++k) {
        const int zz = zb + k;
        const float4 zp = zrow(zz + 1);
        const long long c = c00 + (long long)zz * sz;
        const float4 ym = nyb.wm ? ld4(in, c + nyb.om) : zero4;
        const float4 yp = nyb.wp ? ld4(in, c + nyb.op) : zero4;
        const float4 bv = ld4(b, c);
        const float4 dv = (MODE == 2) ? ld4(dot, c) : zero4;
        const float sl = __shfl_up_sync(0xffffffffu, zc.w, 1);
        const float sr = __shfl_down_sync(0xffffffffu, zc.x, 1);
        const float left = ownl ? mg_ldw_f(in, c + ol, wl) : sl;
        const float right = ownr ? mg_ldw_f(in, c + orr, wr) : sr;
        const int dzw = (int)(zz > 0 || g.per[0]) + (int)(zz < nz - 1 || g.per[0]);
        const float xc[4] = {zc.x, zc.y, zc.z, zc.w};
        const float xm[4] = {left, zc.x, zc.y, zc.z}, xp[4] = {zc.y, zc.z, zc.w, right};
        const float ymv[4] = {ym.x, ym.y, ym.z, ym.w}, ypv[4] = {yp.x, yp.y, yp.z, yp.w};
        const float zmv[4] = {zm.x, zm.y, zm.z, zm.w}, zpv[4] = {zp.x, zp.y, zp.z, zp.w};
        const float bb[4] = {bv.x, bv.y, bv.z, bv.w}, dd[4] = {dv.x, dv.y, dv.z, dv.w};
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float s = ((((xm[e] + xp[e]) + ymv[e]) + ypv[e]) + zmv[e]) + zpv[e];
            v[e] = cff1 * xc[e] + (s - bb[e]) * mg_idiag<float>(g, dgx[e] + dzw);
            if (MODE == 2 && act) {
                sdot = __fmaf_rn(v[e], dd[e], sdot);
                ssum = __fadd_rn(ssum, v[e]);
            }
        }
        if (act) {
            if (MODE == 1) {
                float4* a4 = reinterpret_cast<float4*>(acc + c);
                float4 a01 = a4[0], a23 = a4[1];
                float2 r0 = df_add_f(make_float2(a01.x, a01.y), v[0]), r1 = df_add_f(make_float2(a01.z, a01.w), v[1]);
                float2 r2 = df_add_f(make_float2(a23.x, a23.y), v[2]), r3 = df_add_f(make_float2(a23.z, a23.w), v[3]);
                a4[0] = make_float4(r0.x, r0.y, r1.x, r1.y);
                a4[1] = make_float4(r2.x, r2.y, r3.x, r3.y);
            } else {
                *reinterpret_cast<float4*>(out + c) = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
        zm = zc;
        zc = zp;
    }
}

template <int MODE, bool BAT = false, int ZC = V4_ZC>
__global__ void __launch_bounds__(MG_BX * MG_BY, 5) k_mg_jacobi_v4(const MgGeom g, const float* __restrict__ in,
                                                               const float* __restrict__ b, float* __restrict__ out,
                                                               float omega, float2* __restrict__ acc,
                                                               const float* __restrict__ dot,
                                                               double* __restrict__ partial,
                                                               double* __restrict__ partial2, const Bat bat = Bat(),
                                                               const MgFin fin = MgFin()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        in = bshift(in, dlt);
        b = bshift(b, dlt);
        out = bshift(out, dlt);
        acc = bshift(acc, dlt);
        dot = bshift(dot, dlt);
        partial = bshift(partial, dlt);
        partial2 = bshift(partial2, dlt);
    }
    float sdot = 0.f, ssum = 0.f;
    mg_jacobi_v4_blk<MODE, ZC>(g, in, b, out, omega, acc, dot, blockIdx.x, blockIdx.y, bz, sdot, ssum);
    if constexpr (MODE == 2) {
        block_partial2_f(sdot, ssum, partial, partial2, bz);
        // the Krylov solve's beta and mean of z from the totals (k_fcg_final_beta's work)
        if (!BAT && fin.ticket) {
            const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
            if (mg_last_block(fin.ticket, nblk)) {
                const double2 t = mg_block_total2(partial, partial2, (int)nblk);
                if (threadIdx.x == 0 && threadIdx.y == 0) fcg_set_beta(t.x, t.y, fin.vol, fin.sc, fin.k);
            }
        }
    }
}

// First half-sweep of a level whose solution is zero: (1-omega)*0 + omega*(0-b)*idiag
// depends on the cell's own b alone, so the kernel that produces b writes it.
template <typename T>
__device__ __forceinline__ T mg_jacobi_from_zero(T b, T omega, T idg) {
    (void)omega;   // idg = omega/diag
    return (T(0) - b) * idg;
}

// residual of the fine level restricted to the coarse right-hand side,
// bc = Rcoef*(sum of the 8 children) with Rcoef = 1/2 (basicoperators.f90:32-60,
// operators.f90:172-213). The coarse solution is zero at this point (operators.f90:209),
// so the first half-sweep of the coarse smoothing is written here, into yc.
template <typename T, bool BAT = false>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_restrict(const MgGeom gf, const T* __restrict__ xf,
                                                              const T* __restrict__ bf, const MgGeom gc,
                                                              T* __restrict__ bc, T* __restrict__ yc, T omega,
                                                              const Bat bat = Bat()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        xf = bshift(xf, dlt);
        bf = bshift(bf, dlt);
        bc = bshift(bc, dlt);
        yc = bshift(yc, dlt);
    }
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    if (x >= gc.n[2] || y >= gc.n[1]) return;
    const int nzc = gc.n[0], z0 = bz * MG_RZC;
    auto emit = [&](int z, T s) {
        const long long c = mg_at(gc, z, y, x);
        const T bv = T(0.5) * s;
        bc[c] = bv;
        yc[c] = mg_jacobi_from_zero(bv, omega, mg_idiag<T>(gc, mg_diag(gc, z, y, x)));
    };
    if (z0 + MG_RZC > nzc) {   // last, partial chunk
        for (int z = z0; z < nzc; ++z) emit(z, mg_restrict_cell(gf, xf, bf, z, y, x));
        return;
    }
    // Full chunk, unrolled: the 2 x 2 children of each fine plane 2*z0-1 .. 2*(z0+RZC)
    // and their x/y neighbours are loaded up front; residuals of the children in
    // mgfor's neighbour order, summed in the order (k,j,i), (k,j,i+1), (k,j+1,i),
    // (k,j+1,i+1), then the same at k+1.
    const long long sy = gf.n[2], sz = (long long)gf.n[1] * gf.n[2];
    const int i0 = 2 * x, j0 = 2 * y, k0 = 2 * z0;
    const MgNb xl = mg_nb(i0, gf.n[2], gf.per[2], 1), xh = mg_nb(i0 + 1, gf.n[2], gf.per[2], 1);
    const MgNb yl = mg_nb(j0, gf.n[1], gf.per[1], sy), yh = mg_nb(j0 + 1, gf.n[1], gf.per[1], sy);
    const MgNb zl = mg_nb(k0, gf.n[0], gf.per[0], sz), zh = mg_nb(k0 + 2 * MG_RZC - 1, gf.n[0], gf.per[0], sz);
    // wet x/y neighbours of the children (j0,i0), (j0,i1), (j1,i0), (j1,i1)
    const int dxy[4] = {(int)xl.wm + 1 + (int)yl.wm + 1, 1 + (int)xh.wp + (int)yl.wm + 1,
                        (int)xl.wm + 1 + 1 + (int)yh.wp, 1 + (int)xh.wp + 1 + (int)yh.wp};
    const long long cb = mg_at(gf, k0, j0, i0);
    constexpr int NP = 2 * MG_RZC + 2;   // fine planes k0-1 .. k0+2*RZC
    T v[NP][4];
    auto ld4 = [&](long long c, bool wet, T* o) {
        o[0] = mg_ldw(xf, c, wet);
        o[1] = mg_ldw(xf, c + 1, wet);
        o[2] = mg_ldw(xf, c + sy, wet);
        o[3] = mg_ldw(xf, c + sy + 1, wet);
    };
    ld4(cb + zl.om, zl.wm, v[0]);
#pragma unroll
    for (int q = 1; q < NP - 1; ++q) ld4(cb + (q - 1) * sz, true, v[q]);
    ld4(cb + (2 * MG_RZC - 1) * sz + zh.op, zh.wp, v[NP - 1]);
    // The 8 residuals b + diag*x - sum(x_nb) summed at once: each child's 6 neighbours
    // are 3 siblings and 3 cells outside the 2 x 2 x 2 block, so the sum is
    // sum(b) + sum(w_c x_c) - sum(24 outside cells) with w_c = diag_c - 3, the child's wet
    // outside neighbours (dry ones are read as 0). Same value as the per-child sums up
    // to rounding, with 2/3 of their FP64 instructions.
    const T wxy[4] = {T(dxy[0] - 2), T(dxy[1] - 2), T(dxy[2] - 2), T(dxy[3] - 2)};
#pragma unroll
    for (int zc = 0; zc < MG_RZC; ++zc) {
        T sb = T(0), sx = T(0), so = T(0);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int q = 2 * zc + 1 + h;   // plane index in v
            const long long c = cb + (q - 1) * sz;
            // the plane's z-neighbour outside the block: below for the lower plane, above
            // for the upper one (dry at a closed wall)
            const bool wz = (h == 0) ? (q == 1 ? zl.wm : true) : (q == NP - 2 ? zh.wp : true);
            const T* zo = v[h == 0 ? q - 1 : q + 1];
            // x/y ring of the plane
            const T xm0 = mg_ldw(xf, c + xl.om, xl.wm), xm1 = mg_ldw(xf, c + sy + xl.om, xl.wm);
            const T xp0 = mg_ldw(xf, c + 1 + xh.op, xh.wp), xp1 = mg_ldw(xf, c + sy + 1 + xh.op, xh.wp);
            const T ym0 = mg_ldw(xf, c + yl.om, yl.wm), ym1 = mg_ldw(xf, c + 1 + yl.om, yl.wm);
            const T yp0 = mg_ldw(xf, c + sy + yh.op, yh.wp), yp1 = mg_ldw(xf, c + sy + 1 + yh.op, yh.wp);
            const T* p = v[q];
            sb = sb + ((bf[c] + bf[c + 1]) + (bf[c + sy] + bf[c + sy + 1]));
            const T pp = (p[0] + p[1]) + (p[2] + p[3]);
            sx = sx + (wxy[0] * p[0] + wxy[1] * p[1] + wxy[2] * p[2] + wxy[3] * p[3]);
            sx = wz ? sx + pp : sx;
            so = so + ((((xm0 + xm1) + (xp0 + xp1)) + ((ym0 + ym1) + (yp0 + yp1))) + ((zo[0] + zo[1]) + (zo[2] + zo[3])));
        }
        emit(z0 + zc, (sb + sx) - so);
    }
}

// trilinear 9-3-3-1 prolongation added to the fine solution (basicoperators.f90:173-231)
template <typename T, bool BAT = false>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_prolong(const MgGeom gf, T* __restrict__ xf, const MgGeom gc,
                                                             const T* __restrict__ xc, const Bat bat = Bat()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        xf = bshift(xf, dlt);
        xc = bshift(xc, dlt);
    }
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    if (x >= gf.n[2] || y >= gf.n[1]) return;
    const int nzf = gf.n[0], z0 = bz * MG_ZC;   // z0 even
    if (z0 + MG_ZC > nzf) {   // last, partial chunk
        for (int z = z0; z < nzf; ++z) {
            const long long c = mg_at(gf, z, y, x);
            xf[c] = xf[c] + mg_prolong_cell(gf, gc, xc, z, y, x);
        }
        return;
    }
    // Full chunk, unrolled: the in-plane 9-3-3-1 sums of the coarse planes z0/2-1 ..
    // z0/2+ZC/2 (each used by two fine planes) are formed once; a coarse neighbour
    // outside the level is the periodic image or 0.
    const int ic = x >> 1, jc = y >> 1;
    const long long csy = gc.n[2], csz = (long long)gc.n[1] * gc.n[2];
    const MgNb cx = mg_nb(ic, gc.n[2], gc.per[2], 1), cy = mg_nb(jc, gc.n[1], gc.per[1], csy);
    const long long ox = (x & 1) ? cx.op : cx.om, oy = (y & 1) ? cy.op : cy.om;
    const bool wx = (x & 1) ? cx.wp : cx.wm, wy = (y & 1) ? cy.wp : cy.wm;
    const int kc0 = z0 >> 1;
    const MgNb zl = mg_nb(kc0, gc.n[0], gc.per[0], csz), zh = mg_nb(kc0 + MG_ZC / 2 - 1, gc.n[0], gc.per[0], csz);
    const long long cc = mg_at(gc, kc0, jc, ic);
    auto plane = [&](long long c, bool wet) -> T {
        const T a = mg_ldw(xc, c, wet), b = mg_ldw(xc, c + ox, wet && wx);
        const T d = mg_ldw(xc, c + oy, wet && wy), e = mg_ldw(xc, c + ox + oy, wet && wx && wy);
        return ((T(9) * a + T(3) * b) + T(3) * d) + e;
    };
    const long long c0 = mg_at(gf, z0, y, x), sz = (long long)gf.n[1] * gf.n[2];
    T xv[MG_ZC];   // the fine values, loaded together with the coarse ones
#pragma unroll
    for (int k = 0; k < MG_ZC; ++k) xv[k] = xf[c0 + k * sz];
    constexpr int NP = MG_ZC / 2 + 2;
    T P[NP];
    P[0] = plane(cc + zl.om, zl.wm);
#pragma unroll
    for (int q = 1; q < NP - 1; ++q) P[q] = plane(cc + (q - 1) * csz, true);
    P[NP - 1] = plane(cc + (MG_ZC / 2 - 1) * csz + zh.op, zh.wp);
    const int bxy = (int)wx | ((int)wy << 1);
    const T pc_wet = mg_pcoef<T>(gf, bxy | 4), pc_lo = mg_pcoef<T>(gf, bxy | ((int)zl.wm << 2));
    const T pc_hi = mg_pcoef<T>(gf, bxy | ((int)zh.wp << 2));
#pragma unroll
    for (int k = 0; k < MG_ZC; ++k) {
        const int m = (k >> 1) + 1;                  // plane of z>>1 in P
        const T bpl = P[m], opl = P[(k & 1) ? m + 1 : m - 1];
        const T pc = (k == 0) ? pc_lo : (k == MG_ZC - 1 ? pc_hi : pc_wet);
        xf[c0 + k * sz] = xv[k] + pc * (T(3) * bpl + opl);
    }
}

// Vector forms of the two transfers (FP32): a thread owns 4 consecutive fine x cells,
// i.e. 2 coarse x cells, so that fine rows move as 16-byte and coarse pairs as 8-byte
// accesses; x neighbours come from the adjacent lanes (loaded at the warp's ends and at
// the level's x faces). Idle lanes shadow the last vector of their row so that every
// lane takes part in the shuffles; only active lanes store. Both need the fine level
// twice the coarse one in every direction and fine nx divisible by 4, and keep the
// per-cell arithmetic of the full-chunk paths above.

// k_mg_restrict: one coarse row pair of cells per thread, RZC coarse planes (needs
// coarse nz divisible by RZC); block (bx, by, bz) of the grid grid_v4_restrict(fine, coarse, RZC)
template <int RZC>
__device__ __forceinline__ void mg_restrict_v4_blk(const MgGeom& gf, const float* __restrict__ xf,
                                                   const float* __restrict__ bf, const MgGeom& gc,
                                                   float* __restrict__ bc, float* __restrict__ yc, float omega, int bx,
                                                   int by, int bz) {
    const int nx = gf.n[2], ny = gf.n[1], nz = gf.n[0];
    const int nx4 = nx >> 2;
    const int lane = threadIdx.x;
    const int xv = bx * MG_BX + lane;
    const int jc = by * MG_BY + threadIdx.y;   // coarse row
    const bool act = xv < nx4 && jc < gc.n[1];
    const int x0 = min(xv, nx4 - 1) * 4, j0 = 2 * min(jc, gc.n[1] - 1);
    const long long sy = nx, sz = (long long)ny * nx;
    const MgNb yl = mg_nb(j0, ny, gf.per[1], sy), yh = mg_nb(j0 + 1, ny, gf.per[1], sy);
    const bool wl = x0 > 0 || gf.per[2], wr = x0 + 4 < nx || gf.per[2];
    const long long ol = x0 > 0 ? -1 : (gf.per[2] ? (long long)(nx - 1) : 0);
    const long long orr = x0 + 4 < nx ? 4 : (gf.per[2] ? (long long)(4 - nx) : 0);
    const bool ownl = lane == 0 || x0 == 0, ownr = lane == MG_BX - 1 || x0 + 4 >= nx;
    // w_c = wet outside x/y neighbours of each child (j0,i), (j0,i+1), (j0+1,i), (j0+1,i+1)
    // of the coarse cells m = 0 (fine x0, x0+1) and m = 1 (x0+2, x0+3)
    const int ylw = (int)yl.wm, yhw = (int)yh.wp;
    const float wxy[2][4] = {{(float)((int)wl + ylw), (float)(1 + ylw), (float)((int)wl + yhw), (float)(1 + yhw)},
                             {(float)(1 + ylw), (float)((int)wr + ylw), (float)(1 + yhw), (float)((int)wr + yhw)}};
    const int zcb = bz * RZC, k0 = 2 * zcb;
    const long long c00 = (long long)j0 * sy + x0;
    auto ld4 = [&](const float* a, long long c) { return *reinterpret_cast<const float4*>(a + c); };
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    struct Rows { float4 r0, r1; };
    // rows j0 and j0 + 1 of fine plane k, one plane outside the level at most: periodic
    // image, or 0 across a closed wall
    auto plane = [&](int k) -> Rows {
        Rows R;
        if ((k < 0 || k >= nz) && !gf.per[0]) {
            R.r0 = zero4;
            R.r1 = zero4;
            return R;
        }
        const int kk = k < 0 ? k + nz : (k >= nz ? k - nz : k);
        const long long c = c00 + (long long)kk * sz;
        R.r0 = ld4(xf, c);
        R.r1 = ld4(xf, c + sy);
        return R;
    };
    Rows below = plane(k0 - 1), cur = plane(k0);
#pragma unroll
    for (int zc = 0; zc < RZC; ++zc) {
        const int kz = k0 + 2 * zc;
        const Rows up = plane(kz + 1), nxt = plane(kz + 2);
        float sbv[2] = {0.f, 0.f}, sxv[2] = {0.f, 0.f}, sov[2] = {0.f, 0.f};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int kf = kz + h;
            const Rows& P = h == 0 ? cur : up;
            const Rows& O = h == 0 ? below : nxt;   // the plane's z-neighbour outside the block
            const bool wz = h == 0 ? (kf > 0 || gf.per[0]) : (kf < nz - 1 || gf.per[0]);
            const long long c = c00 + (long long)kf * sz;
            const float4 ym = yl.wm ? ld4(xf, c + yl.om) : zero4;
            const float4 yp = yh.wp ? ld4(xf, c + sy + yh.op) : zero4;
            const float4 b0 = ld4(bf, c), b1 = ld4(bf, c + sy);
            const float sl0 = __shfl_up_sync(0xffffffffu, P.r0.w, 1), sl1 = __shfl_up_sync(0xffffffffu, P.r1.w, 1);
            const float sr0 = __shfl_down_sync(0xffffffffu, P.r0.x, 1), sr1 = __shfl_down_sync(0xffffffffu, P.r1.x, 1);
            const float l0 = ownl ? mg_ldw_f(xf, c + ol, wl) : sl0, l1 = ownl ? mg_ldw_f(xf, c + sy + ol, wl) : sl1;
            const float r0 = ownr ? mg_ldw_f(xf, c + orr, wr) : sr0, r1 = ownr ? mg_ldw_f(xf, c + sy + orr, wr) : sr1;
            const float x0v[4] = {P.r0.x, P.r0.y, P.r0.z, P.r0.w}, x1v[4] = {P.r1.x, P.r1.y, P.r1.z, P.r1.w};
            const float o0[4] = {O.r0.x, O.r0.y, O.r0.z, O.r0.w}, o1[4] = {O.r1.x, O.r1.y, O.r1.z, O.r1.w};
            const float ymv[4] = {ym.x, ym.y, ym.z, ym.w}, ypv[4] = {yp.x, yp.y, yp.z, yp.w};
            const float b0v[4] = {b0.x, b0.y, b0.z, b0.w}, b1v[4] = {b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                const int i = 2 * m;
                const float p[4] = {x0v[i], x0v[i + 1], x1v[i], x1v[i + 1]};
                const float xm0 = m == 0 ? l0 : x0v[1], xm1 = m == 0 ? l1 : x1v[1];
                const float xp0 = m == 0 ? x0v[2] : r0, xp1 = m == 0 ? x1v[2] : r1;
                sbv[m] = sbv[m] + ((b0v[i] + b0v[i + 1]) + (b1v[i] + b1v[i + 1]));
                const float pp = (p[0] + p[1]) + (p[2] + p[3]);
                sxv[m] = sxv[m] + (wxy[m][0] * p[0] + wxy[m][1] * p[1] + wxy[m][2] * p[2] + wxy[m][3] * p[3]);
                sxv[m] = wz ? sxv[m] + pp : sxv[m];
                sov[m] = sov[m] + ((((xm0 + xm1) + (xp0 + xp1)) + ((ymv[i] + ymv[i + 1]) + (ypv[i] + ypv[i + 1]))) +
                                   ((o0[i] + o0[i + 1]) + (o1[i] + o1[i + 1])));
            }
        }
        if (act) {
            const int z = zcb + zc, xc0 = x0 >> 1;
            const long long cc = mg_at(gc, z, jc, xc0);
            float bv[2], yv[2];
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                bv[m] = 0.5f * ((sbv[m] + sxv[m]) - sov[m]);
                yv[m] = mg_jacobi_from_zero(bv[m], omega, mg_idiag<float>(gc, mg_diag(gc, z, jc, xc0 + m)));
            }
            *reinterpret_cast<float2*>(bc + cc) = make_float2(bv[0], bv[1]);
            *reinterpret_cast<float2*>(yc + cc) = make_float2(yv[0], yv[1]);
        }
        below = up;
        cur = nxt;
    }
}

template <bool BAT = false, int RZC = MG_RZC>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_restrict_v4(const MgGeom gf, const float* __restrict__ xf,
                                                                 const float* __restrict__ bf, const MgGeom gc,
                                                                 float* __restrict__ bc, float* __restrict__ yc,
                                                                 float omega, const Bat bat = Bat()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        xf = bshift(xf, dlt);
        bf = bshift(bf, dlt);
        bc = bshift(bc, dlt);
        yc = bshift(yc, dlt);
    }
    mg_restrict_v4_blk<RZC>(gf, xf, bf, gc, bc, yc, omega, blockIdx.x, blockIdx.y, bz);
}

// k_mg_prolong: one 4-cell fine row segment per thread, ZC fine planes (needs fine nz
// divisible by ZC, ZC even); block (bx, by, bz) of the grid grid_v4(fine n, ZC)
template <int ZC>
__device__ __forceinline__ void mg_prolong_v4_blk(const MgGeom& gf, float* __restrict__ xf, const MgGeom& gc,
                                                  const float* __restrict__ xc, int bx, int by, int bz) {
    const int nx = gf.n[2], ny = gf.n[1];
    const int nx4 = nx >> 2;
    const int lane = threadIdx.x;
    const int xv = bx * MG_BX + lane;
    const int y = by * MG_BY + threadIdx.y;
    const bool act = xv < nx4 && y < ny;
    const int x0 = min(xv, nx4 - 1) * 4, ys = min(y, ny - 1);
    const int ncx = gc.n[2], ic0 = x0 >> 1, jc = ys >> 1;
    const long long csy = ncx, csz = (long long)gc.n[1] * ncx;
    const MgNb cy = mg_nb(jc, gc.n[1], gc.per[1], csy);
    const long long oy = (ys & 1) ? cy.op : cy.om;
    const bool wy = (ys & 1) ? cy.wp : cy.wm;
    // coarse x neighbours of the pair ic0, ic0 + 1: ic0 - 1 (fine x0) and ic0 + 2 (x0 + 3)
    const bool cwl = ic0 > 0 || gc.per[2], cwr = ic0 + 2 < ncx || gc.per[2];
    const long long col = ic0 > 0 ? -1 : (gc.per[2] ? (long long)(ncx - 1) : 0);
    const long long cor = ic0 + 2 < ncx ? 2 : (gc.per[2] ? (long long)(2 - ncx) : 0);
    const bool ownl = lane == 0 || x0 == 0, ownr = lane == MG_BX - 1 || x0 + 4 >= nx;
    const int zb = bz * ZC, kc0 = zb >> 1;
    const MgNb zl = mg_nb(kc0, gc.n[0], gc.per[0], csz), zh = mg_nb(kc0 + ZC / 2 - 1, gc.n[0], gc.per[0], csz);
    const long long cc = mg_at(gc, kc0, jc, ic0);
    // in-plane 9-3-3-1 sums of the 4 fine cells from one coarse plane at c (0 when the
    // plane is dry): fine x0 + e takes coarse ic0 + (e >> 1) and its x neighbour on the
    // side of the fine cell
    auto plane = [&](long long c, bool wet, float* out) {
        const float2 a = wet ? *reinterpret_cast<const float2*>(xc + c) : make_float2(0.f, 0.f);
        const float2 d = (wet && wy) ? *reinterpret_cast<const float2*>(xc + c + oy) : make_float2(0.f, 0.f);
        const float sal = __shfl_up_sync(0xffffffffu, a.y, 1), sar = __shfl_down_sync(0xffffffffu, a.x, 1);
        const float sdl = __shfl_up_sync(0xffffffffu, d.y, 1), sdr = __shfl_down_sync(0xffffffffu, d.x, 1);
        const float al = ownl ? mg_ldw_f(xc, c + col, wet && cwl) : sal;
        const float ar = ownr ? mg_ldw_f(xc, c + cor, wet && cwr) : sar;
        const float dl = ownl ? mg_ldw_f(xc, c + oy + col, wet && cwl && wy) : sdl;
        const float dr = ownr ? mg_ldw_f(xc, c + oy + cor, wet && cwr && wy) : sdr;
        const float av[4] = {a.x, a.x, a.y, a.y}, bv[4] = {al, a.y, a.x, ar};
        const float dv[4] = {d.x, d.x, d.y, d.y}, ev[4] = {dl, d.y, d.x, dr};
#pragma unroll
        for (int e = 0; e < 4; ++e) out[e] = ((9.f * av[e] + 3.f * bv[e]) + 3.f * dv[e]) + ev[e];
    };
    const long long sz = (long long)ny * nx, c0 = (long long)zb * sz + (long long)ys * nx + x0;
    float4 xv4[ZC];   // the fine values, loaded together with the coarse ones
#pragma unroll
    for (int k = 0; k < ZC; ++k) xv4[k] = *reinterpret_cast<const float4*>(xf + c0 + k * sz);
    constexpr int NP = ZC / 2 + 2;
    float P[NP][4];
    plane(cc + zl.om, zl.wm, P[0]);
#pragma unroll
    for (int q = 1; q < NP - 1; ++q) plane(cc + (q - 1) * csz, true, P[q]);
    plane(cc + (ZC / 2 - 1) * csz + zh.op, zh.wp, P[NP - 1]);
    // 1/(Wx*Wy*Wz) of each fine cell: its coarse x neighbour is wet except beyond the
    // level's x faces (cells x0 and x0 + 3)
    float pc_wet[4], pc_lo[4], pc_hi[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const bool wx = e == 0 ? cwl : (e == 3 ? cwr : true);
        const int bxy = (int)wx | ((int)wy << 1);
        pc_wet[e] = mg_pcoef<float>(gf, bxy | 4);
        pc_lo[e] = mg_pcoef<float>(gf, bxy | ((int)zl.wm << 2));
        pc_hi[e] = mg_pcoef<float>(gf, bxy | ((int)zh.wp << 2));
    }
#pragma unroll
    for (int k = 0; k < ZC; ++k) {
        const int m = (k >> 1) + 1;   // plane of z >> 1 in P
        const float* bpl = P[m];
        const float* opl = P[(k & 1) ? m + 1 : m - 1];
        const float xo[4] = {xv4[k].x, xv4[k].y, xv4[k].z, xv4[k].w};
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float pc = (k == 0) ? pc_lo[e] : (k == ZC - 1 ? pc_hi[e] : pc_wet[e]);
            v[e] = xo[e] + pc * (3.f * bpl[e] + opl[e]);
        }
        if (act) *reinterpret_cast<float4*>(xf + c0 + k * sz) = make_float4(v[0], v[1], v[2], v[3]);
    }
}

template <bool BAT = false, int ZC = V4_ZC>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_prolong_v4(const MgGeom gf, float* __restrict__ xf,
                                                                const MgGeom gc, const float* __restrict__ xc,
                                                                const Bat bat = Bat()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        xf = bshift(xf, dlt);
        xc = bshift(xc, dlt);
    }
    mg_prolong_v4_blk<ZC>(gf, xf, gc, xc, blockIdx.x, blockIdx.y, bz);
}

// ---------------------------------------------------------------- coarse levels in one block
// Levels l0..L-1 of a V-cycle (solvers.f90:35-55 from level l0 down and back up) run in
// one thread block: the level arrays live in shared memory, and each half-sweep,
// restriction and prolongation is one pass of the block over a level followed by a
// barrier, instead of one grid launch each. Input: b of level l0 (its x is zero after
// the restriction that produced b); output: x of level l0. The per-cell arithmetic is
// that of the grid kernels' ghost paths.
constexpr int MG_BOTTOM_MAXLEV = 12;
constexpr size_t MG_BOTTOM_SMEM = 200 * 1024;
constexpr long long MG_BOTTOM_MAXVOL_FP64 = 1024;   // largest level (cells) in the FP64 one-block kernel
template <typename T> struct MgBottomThreads { static constexpr int n = 1024; };
template <> struct MgBottomThreads<double> { static constexpr int n = 512; };   // register budget

template <typename T>
struct MgBottom {
    int nlev;                          // levels held: l0..L-1
    MgGeom g[MG_BOTTOM_MAXLEV];
    int off[MG_BOTTOM_MAXLEV];         // element offset of each level's x in shared memory; b, y follow
    T* xg;                             // x of level l0 (global)
    const T* bg;                       // b of level l0 (global)
    T omega;
};

__device__ __forceinline__ int mg_vol(const MgGeom& g) { return g.n[0] * g.n[1] * g.n[2]; }

// neighbours along one direction with 32-bit offsets (levels held in shared memory)
struct MgNbI {
    int om, op;
    bool wm, wp;
};
__device__ __forceinline__ MgNbI mg_nbi(int c, int n, int per, int stride) {
    MgNbI r;
    r.wm = c > 0 || per;
    r.wp = c < n - 1 || per;
    r.om = c > 0 ? -stride : (per ? (n - 1) * stride : 0);
    r.op = c < n - 1 ? stride : (per ? -(n - 1) * stride : 0);
    return r;
}
template <typename T>
__device__ __forceinline__ T sm_ldw(const T* a, int c, bool wet) {
    const T v = a[c];
    return wet ? v : T(0);
}

// Visit every cell of a level: threads take (x, y) columns, split in z when the block
// has more threads than the level has columns; f(z, y, x, nx, ny) gets the column's
// x/y neighbours.
template <typename F>
__device__ __forceinline__ void bottom_cells(const MgGeom& g, F f) {
    const int ncol = g.n[1] * g.n[2], nz = g.n[0];
    if (ncol == 0 || nz == 0) return;
    const int groups = max(1, (int)blockDim.x / ncol);
    const int zc = (nz + groups - 1) / groups;
    // power-of-two extents (the usual coarse levels): masks and shifts instead of the
    // integer divisions, which took a large share of a pass over a small level
    const int n2 = g.n[2];
    const bool p2 = ((ncol & (ncol - 1)) | (n2 & (n2 - 1))) == 0;
    const int lc = __ffs(ncol) - 1, l2 = __ffs(n2) - 1;
    for (int t = threadIdx.x; t < ncol * groups; t += blockDim.x) {
        int col, grp, x, y;
        if (p2) {
            col = t & (ncol - 1);
            grp = t >> lc;
            x = col & (n2 - 1);
            y = col >> l2;
        } else {
            col = t % ncol;
            grp = t / ncol;
            x = col % n2;
            y = col / n2;
        }
        const MgNbI nx = mg_nbi(x, g.n[2], g.per[2], 1), ny = mg_nbi(y, g.n[1], g.per[1], g.n[2]);
        const int ze = min(nz, (grp + 1) * zc);
        for (int z = grp * zc; z < ze; ++z) f(z, y, x, nx, ny);
    }
}

// one half-sweep in -> out over a level held in shared memory
template <typename T>
__device__ __forceinline__ void bottom_sweep(const MgGeom& g, const T* in, const T* b, T* out, T cff1, T om) {
    const int sz = g.n[1] * g.n[2];
    bottom_cells(g, [&](int z, int y, int x, const MgNbI& nx, const MgNbI& ny) {
        const int c = (z * g.n[1] + y) * g.n[2] + x;
        const MgNbI nzb = mg_nbi(z, g.n[0], g.per[0], sz);
        const T idg = mg_idiag<T>(g, (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp + (int)nzb.wm + (int)nzb.wp);
        const T s = ((((sm_ldw(in, c + nx.om, nx.wm) + sm_ldw(in, c + nx.op, nx.wp)) + sm_ldw(in, c + ny.om, ny.wm)) +
                      sm_ldw(in, c + ny.op, ny.wp)) + sm_ldw(in, c + nzb.om, nzb.wm)) + sm_ldw(in, c + nzb.op, nzb.wp);
        out[c] = cff1 * in[c] + (s - b[c]) * idg;
    });
    __syncthreads();
}

// 1/diag of a cell from its column's x/y neighbours and its z position
template <typename T>
__device__ __forceinline__ T bottom_idiag(const MgGeom& g, int z, const MgNbI& nx, const MgNbI& ny) {
    const MgNbI nzb = mg_nbi(z, g.n[0], g.per[0], 0);
    return mg_idiag<T>(g, (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp + (int)nzb.wm + (int)nzb.wp);
}

// sum of the residuals of the 8 children of coarse cell (z, y, x), shared-memory level
// (mg_restrict_cell with direct neighbour offsets)
template <typename T>
__device__ __forceinline__ T bottom_restrict(const MgGeom& gf, const T* xf, const T* bf, int z, int y, int x) {
    const int nx = gf.n[2], ny = gf.n[1], nz = gf.n[0], sy = nx, sz = nx * ny;
    const int i0 = 2 * x, j0 = 2 * y, k0 = 2 * z;
    const MgNbI xl = mg_nbi(i0, nx, gf.per[2], 1), xh = mg_nbi(i0 + 1, nx, gf.per[2], 1);
    const MgNbI yl = mg_nbi(j0, ny, gf.per[1], sy), yh = mg_nbi(j0 + 1, ny, gf.per[1], sy);
    const MgNbI zl = mg_nbi(k0, nz, gf.per[0], sz), zh = mg_nbi(k0 + 1, nz, gf.per[0], sz);
    const int dxy[4] = {(int)xl.wm + 1 + (int)yl.wm + 1, 1 + (int)xh.wp + (int)yl.wm + 1,
                        (int)xl.wm + 1 + 1 + (int)yh.wp, 1 + (int)xh.wp + 1 + (int)yh.wp};
    const int cb = (k0 * ny + j0) * nx + i0;
    T v[4][4];   // the 2 x 2 children positions on planes k0-1 .. k0+2
    auto ld4 = [&](int c, bool wet, T* o) {
        o[0] = sm_ldw(xf, c, wet);
        o[1] = sm_ldw(xf, c + 1, wet);
        o[2] = sm_ldw(xf, c + sy, wet);
        o[3] = sm_ldw(xf, c + sy + 1, wet);
    };
    ld4(cb + zl.om, zl.wm, v[0]);
    ld4(cb, true, v[1]);
    ld4(cb + sz, true, v[2]);
    ld4(cb + sz + zh.op, zh.wp, v[3]);
    T s = T(0);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int q = h + 1;
        const int c = cb + h * sz;
        const int dz = (h == 0 ? (int)zl.wm : 1) + (h == 1 ? (int)zh.wp : 1);
        const T xm0 = sm_ldw(xf, c + xl.om, xl.wm), xm1 = sm_ldw(xf, c + sy + xl.om, xl.wm);
        const T xp0 = sm_ldw(xf, c + 1 + xh.op, xh.wp), xp1 = sm_ldw(xf, c + sy + 1 + xh.op, xh.wp);
        const T ym0 = sm_ldw(xf, c + yl.om, yl.wm), ym1 = sm_ldw(xf, c + 1 + yl.om, yl.wm);
        const T yp0 = sm_ldw(xf, c + sy + yh.op, yh.wp), yp1 = sm_ldw(xf, c + sy + 1 + yh.op, yh.wp);
        const T* p = v[q];
        const T r00 = (bf[c] + T(dxy[0] + dz) * p[0]) - (((((xm0 + p[1]) + ym0) + p[2]) + v[q - 1][0]) + v[q + 1][0]);
        const T r01 = (bf[c + 1] + T(dxy[1] + dz) * p[1]) -
                      (((((p[0] + xp0) + ym1) + p[3]) + v[q - 1][1]) + v[q + 1][1]);
        const T r10 = (bf[c + sy] + T(dxy[2] + dz) * p[2]) -
                      (((((xm1 + p[3]) + p[0]) + yp0) + v[q - 1][2]) + v[q + 1][2]);
        const T r11 = (bf[c + sy + 1] + T(dxy[3] + dz) * p[3]) -
                      (((((p[2] + xp1) + p[1]) + yp1) + v[q - 1][3]) + v[q + 1][3]);
        s = (h == 0) ? r00 : s + r00;
        s = s + r01;
        s = s + r10;
        s = s + r11;
    }
    return s;
}

// prolongation increment of fine cell (z, y, x) from a shared-memory coarse level
// (mg_prolong_cell with direct neighbour offsets)
template <typename T>
__device__ __forceinline__ T bottom_prolong(const MgGeom& gf, const MgGeom& gc, const T* xc, int z, int y, int x) {
    const int ic = x >> 1, jc = y >> 1, kc = z >> 1;
    const int csy = gc.n[2], csz = gc.n[1] * gc.n[2];
    const MgNbI cx = mg_nbi(ic, gc.n[2], gc.per[2], 1), cy = mg_nbi(jc, gc.n[1], gc.per[1], csy);
    const MgNbI cz = mg_nbi(kc, gc.n[0], gc.per[0], csz);
    const int ox = (x & 1) ? cx.op : cx.om, oy = (y & 1) ? cy.op : cy.om, oz = (z & 1) ? cz.op : cz.om;
    const bool wx = (x & 1) ? cx.wp : cx.wm, wy = (y & 1) ? cy.wp : cy.wm, wz = (z & 1) ? cz.wp : cz.wm;
    const int c0 = (kc * gc.n[1] + jc) * gc.n[2] + ic;
    auto plane = [&](int c, bool w) -> T {
        const T a = sm_ldw(xc, c, w), b = sm_ldw(xc, c + ox, w && wx);
        const T d = sm_ldw(xc, c + oy, w && wy), e = sm_ldw(xc, c + ox + oy, w && wx && wy);
        return ((T(9) * a + T(3) * b) + T(3) * d) + e;
    };
    const T bpl = plane(c0, true), opl = plane(c0 + oz, wz);
    const T pcoef = mg_pcoef<T>(gf, (int)wx | ((int)wy << 1) | ((int)wz << 2));
    return pcoef * (T(3) * bpl + opl);
}

template <typename T>
__global__ void __launch_bounds__(MgBottomThreads<T>::n, 1) k_mg_bottom(const MgBottom<T> a, const Bat bat = Bat()) {
    extern __shared__ __align__(16) unsigned char mg_smem[];
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    // the arguments stay in parameter space (their level table is indexed at run time:
    // a copy of the struct would sit in every thread's local memory); only the two
    // global pointers are shifted to the block's run
    T* const xg = bshift(a.xg, dlt);
    const T* const bg = bshift(a.bg, dlt);
    T* sm = reinterpret_cast<T*>(mg_smem);
    const T om = a.omega, cff1 = T(1) - om;
    const int L = a.nlev;
    auto X = [&](int l) { return sm + a.off[l]; };
    auto Bv = [&](int l) { return sm + a.off[l] + mg_vol(a.g[l]); };
    auto Y = [&](int l) { return sm + a.off[l] + 2 * mg_vol(a.g[l]); };
    // level l0 starts from x = 0: its first half-sweep is y = from_zero(b)
    bottom_cells(a.g[0], [&](int z, int y, int x, const MgNbI& nx, const MgNbI& ny) {
        const int c = (z * a.g[0].n[1] + y) * a.g[0].n[2] + x;
        const T bv = bg[c];
        Bv(0)[c] = bv;
        Y(0)[c] = mg_jacobi_from_zero(bv, om, bottom_idiag<T>(a.g[0], z, nx, ny));
    });
    __syncthreads();
    for (int l = 0; l < L - 1; ++l) {
        if (mg_vol(a.g[l]) == 0) break;
        bottom_sweep(a.g[l], Y(l), Bv(l), X(l), cff1, om);   // second half of the pre-smoothing
        const MgGeom& gc = a.g[l + 1];
        if (mg_vol(gc) == 0) break;
        // restriction; the coarse level starts from zero, so its first half-sweep is written too
        bottom_cells(gc, [&](int z, int y, int x, const MgNbI& nx, const MgNbI& ny) {
            const int c = (z * gc.n[1] + y) * gc.n[2] + x;
            const T bv = T(0.5) * bottom_restrict(a.g[l], X(l), Bv(l), z, y, x);
            Bv(l + 1)[c] = bv;
            Y(l + 1)[c] = mg_jacobi_from_zero(bv, om, bottom_idiag<T>(gc, z, nx, ny));
        });
        __syncthreads();
    }
    if (mg_vol(a.g[L - 1]) > 0) bottom_sweep(a.g[L - 1], Y(L - 1), Bv(L - 1), X(L - 1), cff1, om);
    for (int l = L - 2; l >= 0; --l) {
        const MgGeom& gf = a.g[l];
        if (mg_vol(gf) == 0) continue;
        if (mg_vol(a.g[l + 1]) > 0) {
            bottom_cells(gf, [&](int z, int y, int x, const MgNbI&, const MgNbI&) {
                const int c = (z * gf.n[1] + y) * gf.n[2] + x;
                X(l)[c] = X(l)[c] + bottom_prolong(gf, a.g[l + 1], X(l + 1), z, y, x);
            });
            __syncthreads();
        }
        bottom_sweep(gf, X(l), Bv(l), Y(l), cff1, om);
        bottom_sweep(gf, Y(l), Bv(l), X(l), cff1, om);
    }
    const int v0 = mg_vol(a.g[0]);
    for (int q = threadIdx.x; q < v0; q += blockDim.x) xg[q] = X(0)[q];
}

// ---------------------------------------------------------------- reductions
// Deterministic sums: one partial per block of the (x, y, z-chunk) grid, then one
// block adds the partials in a fixed order.

// MODE 0: sum v^2 ; MODE 1: sum r^2 with r = b + diag*x - sum(x_nb)
template <typename T, int MODE>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_sumsq(const MgGeom g, const T* __restrict__ v,
                                                           const T* __restrict__ b, double* __restrict__ partial) {
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const int nz = g.n[0], z0 = blockIdx.z * MG_ZC;
    double s = 0.0;
    if (x < g.n[2] && y < g.n[1]) {
        const long long sy = g.n[2], sz = (long long)g.n[1] * g.n[2];
        const long long c0 = mg_at(g, z0, y, x);
        if (MODE == 0) {
            for (int z = z0; z < min(z0 + MG_ZC, nz); ++z) {
                const double r = (double)v[c0 + (z - z0) * sz];
                s += r * r;
            }
        } else {
            const MgNb nx = mg_nb(x, g.n[2], g.per[2], 1), ny = mg_nb(y, g.n[1], g.per[1], sy);
            const int dxy = (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp;
            auto res = [&](long long c, T zm, T x0, T zp, T dg) -> T {
                return (b[c] + dg * x0) - (((((mg_ldw(v, c + nx.om, nx.wm) + mg_ldw(v, c + nx.op, nx.wp)) +
                                              mg_ldw(v, c + ny.om, ny.wm)) + mg_ldw(v, c + ny.op, ny.wp)) + zm) + zp);
            };
            if (z0 + MG_ZC <= nz) {
                const MgNb lo = mg_nb(z0, nz, g.per[0], sz), hi = mg_nb(z0 + MG_ZC - 1, nz, g.per[0], sz);
                T col[MG_ZC + 2];
                col[0] = mg_ldw(v, c0 + lo.om, lo.wm);
#pragma unroll
                for (int k = 1; k <= MG_ZC; ++k) col[k] = v[c0 + (k - 1) * sz];
                col[MG_ZC + 1] = mg_ldw(v, c0 + (MG_ZC - 1) * sz + hi.op, hi.wp);
                const T d_mid = T(dxy + 2), d_lo = T(dxy + 1 + (int)lo.wm), d_hi = T(dxy + 1 + (int)hi.wp);
#pragma unroll
                for (int k = 0; k < MG_ZC; ++k) {
                    const double r = (double)res(c0 + k * sz, col[k], col[k + 1], col[k + 2],
                                                 k == 0 ? d_lo : (k == MG_ZC - 1 ? d_hi : d_mid));
                    s += r * r;
                }
            } else {
                for (int z = z0; z < nz; ++z) {
                    const long long c = c0 + (z - z0) * sz;
                    const MgNb nzb = mg_nb(z, nz, g.per[0], sz);
                    const double r = (double)res(c, mg_ldw(v, c + nzb.om, nzb.wm), v[c], mg_ldw(v, c + nzb.op, nzb.wp),
                                                 T(dxy + (int)nzb.wm + (int)nzb.wp));
                    s += r * r;
                }
            }
        }
    }
    block_partial(s, partial, blockIdx.z);
}

// Stop-test residual of the level-1 solution together with the first half-sweep of the
// next V-cycle: both need the same neighbour sum, so one pass gives sum(r^2) (same
// partials, same order as k_mg_sumsq MODE 1) and y = (1-omega)*x + omega*(sum - b)*idiag.
// If the solve then stops, y is simply not used.
template <typename T>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_resid_sweep(const MgGeom g, const T* __restrict__ v,
                                                                 const T* __restrict__ b, T* __restrict__ y_out,
                                                                 T omega, double* __restrict__ partial) {
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const int nz = g.n[0], z0 = blockIdx.z * MG_ZC;
    (void)omega;   // the tables hold omega/diag
    double s = 0.0;
    if (x < g.n[2] && y < g.n[1]) {
        const long long sy = g.n[2], sz = (long long)g.n[1] * g.n[2];
        const long long c0 = mg_at(g, z0, y, x);
        const MgNb nx = mg_nb(x, g.n[2], g.per[2], 1), ny = mg_nb(y, g.n[1], g.per[1], sy);
        const int dxy = (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp;
        auto cell = [&](long long c, T zm, T x0, T zp, int dg) {
            const T nsum = ((((mg_ldw(v, c + nx.om, nx.wm) + mg_ldw(v, c + nx.op, nx.wp)) + mg_ldw(v, c + ny.om, ny.wm)) +
                             mg_ldw(v, c + ny.op, ny.wp)) + zm) + zp;
            const T bv = b[c];
            const T r = (bv + T(dg) * x0) - nsum;
            s += (double)r * (double)r;
            // (1-omega)x + omega(nsum - b)/diag = x - (omega/diag) r
            y_out[c] = x0 - mg_idiag<T>(g, dg) * r;
        };
        if (z0 + MG_ZC <= nz) {
            const MgNb lo = mg_nb(z0, nz, g.per[0], sz), hi = mg_nb(z0 + MG_ZC - 1, nz, g.per[0], sz);
            T col[MG_ZC + 2];
            col[0] = mg_ldw(v, c0 + lo.om, lo.wm);
#pragma unroll
            for (int k = 1; k <= MG_ZC; ++k) col[k] = v[c0 + (k - 1) * sz];
            col[MG_ZC + 1] = mg_ldw(v, c0 + (MG_ZC - 1) * sz + hi.op, hi.wp);
#pragma unroll
            for (int k = 0; k < MG_ZC; ++k)
                cell(c0 + k * sz, col[k], col[k + 1], col[k + 2],
                     dxy + (k == 0 ? 1 + (int)lo.wm : (k == MG_ZC - 1 ? 1 + (int)hi.wp : 2)));
        } else {
            for (int z = z0; z < nz; ++z) {
                const long long c = c0 + (z - z0) * sz;
                const MgNb nzb = mg_nb(z, nz, g.per[0], sz);
                cell(c, mg_ldw(v, c + nzb.om, nzb.wm), v[c], mg_ldw(v, c + nzb.op, nzb.wp),
                     dxy + (int)nzb.wm + (int)nzb.wp);
            }
        }
    }
    block_partial(s, partial, blockIdx.z);
}

// ---------------------------------------------------------------- mixed precision
// Float-pair residual r = b + diag*p - sum(p_nb), neighbours in mgfor's order. The
// neighbour sum and the centre product are error-free (TwoSum chain, TwoProduct); the
// rounding errors and the low parts are added last, so r keeps ~2^-48 of the size of
// the cancelling terms before its final rounding to float.
__device__ __forceinline__ float df_resid(float2 bc, float2 pc, float dg, const float2* nb) {
    float s, e, t;
    two_sum(nb[0].x, nb[1].x, s, e);
#pragma unroll
    for (int k = 2; k < 6; ++k) {
        two_sum(s, nb[k].x, s, t);
        e = __fadd_rn(e, t);
    }
    float lo = nb[0].y;
#pragma unroll
    for (int k = 1; k < 6; ++k) lo = __fadd_rn(lo, nb[k].y);
    float c, ce;
    two_prod(dg, pc.x, c, ce);
    float a1, t1, a2, t2;
    two_sum(bc.x, c, a1, t1);
    two_sum(a1, -s, a2, t2);
    const float rest = __fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(bc.y, ce), t1), t2), __fmul_rn(dg, pc.y)),
                                 __fadd_rn(e, lo));
    return __fadd_rn(a2, rest);
}

// float-pair neighbour read with the wet flag of mg_nb (always loads, 0 when dry)
__device__ __forceinline__ float2 mg_ldw_df(const float2* __restrict__ a, long long c, bool wet) {
    const float2 v = a[c];
    return wet ? v : make_float2(0.f, 0.f);
}

// residual of the float-pair solution: its sum of squares (for the stop test), the
// float right-hand side r32 of the next correction V-cycle, and the first half-sweep
// of that V-cycle from its zero initial correction, y32. The squares are summed in
// float per thread on r * scale, scale = sc[SC_SCALE] a power of two near 1/rms(b)
// (k_mg_scale), so that they neither underflow nor overflow; each block partial is
// unscaled in double.
template <bool BAT = false>
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_resid_df(const MgGeom g, const float2* __restrict__ p,
                                                                 const float2* __restrict__ b, float* __restrict__ r32,
                                                                 float* __restrict__ y32, float omega,
                                                                 const double* __restrict__ sc,
                                                                 double* __restrict__ partial, const Bat bat = Bat()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        p = bshift(p, dlt);
        b = bshift(b, dlt);
        r32 = bshift(r32, dlt);
        y32 = bshift(y32, dlt);
        sc = bshift(sc, dlt);
        partial = bshift(partial, dlt);
    }
    constexpr int ZC = MG_DFZC;
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const int nz = g.n[0], z0 = bz * ZC;
    const float scale = (float)sc[SC_SCALE];
    float s = 0.f;
    if (x < g.n[2] && y < g.n[1]) {
        const long long sy = g.n[2], sz = (long long)g.n[1] * g.n[2];
        const MgNb nx = mg_nb(x, g.n[2], g.per[2], 1), ny = mg_nb(y, g.n[1], g.per[1], sy);
        const int dxy = (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp;
        const long long c0 = mg_at(g, z0, y, x);
        // bc: the cell's right-hand side (loaded ahead by the caller)
        auto cell = [&](long long c, float2 zm, float2 p0, float2 zp, int dg, float2 bc) {
            const float2 nb[6] = {mg_ldw_df(p, c + nx.om, nx.wm), mg_ldw_df(p, c + nx.op, nx.wp),
                                  mg_ldw_df(p, c + ny.om, ny.wm), mg_ldw_df(p, c + ny.op, ny.wp), zm, zp};
            const float r = df_resid(bc, p0, (float)dg, nb);
            r32[c] = r;
            y32[c] = mg_jacobi_from_zero(r, omega, mg_idiag<float>(g, dg));
            const float rs = __fmul_rn(r, scale);
            s = __fmaf_rn(rs, rs, s);
        };
        if (z0 + ZC <= nz) {
            const MgNb lo = mg_nb(z0, nz, g.per[0], sz), hi = mg_nb(z0 + ZC - 1, nz, g.per[0], sz);
            float2 col[ZC + 2];
            col[0] = mg_ldw_df(p, c0 + lo.om, lo.wm);
#pragma unroll
            for (int k = 1; k <= ZC; ++k) col[k] = p[c0 + (k - 1) * sz];
            col[ZC + 1] = mg_ldw_df(p, c0 + (ZC - 1) * sz + hi.op, hi.wp);
            float2 bcol[ZC];
#pragma unroll
            for (int k = 0; k < ZC; ++k) bcol[k] = b[c0 + k * sz];
#pragma unroll
            for (int k = 0; k < ZC; ++k)
                cell(c0 + k * sz, col[k], col[k + 1], col[k + 2],
                     dxy + (k == 0 ? 1 + (int)lo.wm : (k == ZC - 1 ? 1 + (int)hi.wp : 2)), bcol[k]);
        } else {
            for (int z = z0; z < nz; ++z) {
                const long long c = c0 + (z - z0) * sz;
                const MgNb nzb = mg_nb(z, nz, g.per[0], sz);
                cell(c, mg_ldw_df(p, c + nzb.om, nzb.wm), p[c], mg_ldw_df(p, c + nzb.op, nzb.wp),
                     dxy + (int)nzb.wm + (int)nzb.wp, b[c]);
            }
        }
    }
    block_partial_f(s, sc[SC_INVSCALE2], partial, bz);
}

// k_mg_resid_df with 4 consecutive x cells per thread: each float-pair row segment is
// two 16-byte loads, the x neighbours come from the adjacent lanes (loaded at the warp's
// ends and at the level's x faces), r32 and y32 are stored 16 bytes at a time. Needs nx
// and nz divisible by 4 and V4_ZC; same per-cell arithmetic as k_mg_resid_df.
struct DfVec4 {
    float2 v[4];
};
template <bool BAT = false>
__global__ void __launch_bounds__(MG_BX * MG_BY, 3) k_mg_resid_df_v4(const MgGeom g, const float2* __restrict__ p,
                                                                    const float2* __restrict__ b,
                                                                    float* __restrict__ r32, float* __restrict__ y32,
                                                                    float omega, const double* __restrict__ sc,
                                                                    double* __restrict__ partial,
                                                                    const Bat bat = Bat(), MgFin fin = MgFin()) {
    int bz = blockIdx.z;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        p = bshift(p, dlt);
        b = bshift(b, dlt);
        r32 = bshift(r32, dlt);
        y32 = bshift(y32, dlt);
        sc = bshift(sc, dlt);
        partial = bshift(partial, dlt);
        fin.ticket = bshift(fin.ticket, dlt);
        fin.sc = bshift(fin.sc, dlt);
    }
    const int nx = g.n[2], ny = g.n[1], nz = g.n[0];
    const int nx4 = nx >> 2;
    const int lane = threadIdx.x;
    const int xv = blockIdx.x * MG_BX + lane;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const float scale = (float)sc[SC_SCALE];
    float s = 0.f;
    const bool act = xv < nx4 && y < ny;
    const int x0 = min(xv, nx4 - 1) * 4, ys = min(y, ny - 1);
    const long long sy = nx, sz = (long long)ny * nx;
    const MgNb nyb = mg_nb(ys, ny, g.per[1], sy);
    const bool wl = x0 > 0 || g.per[2], wr = x0 + 4 < nx || g.per[2];
    const long long ol = x0 > 0 ? -1 : (g.per[2] ? (long long)(nx - 1) : 0);
    const long long orr = x0 + 4 < nx ? 4 : (g.per[2] ? (long long)(4 - nx) : 0);
    const bool ownl = lane == 0 || x0 == 0, ownr = lane == MG_BX - 1 || x0 + 4 >= nx;
    int dgx[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int xx = x0 + e;
        dgx[e] = (int)(xx > 0 || g.per[2]) + (int)(xx < nx - 1 || g.per[2]) + (int)nyb.wm + (int)nyb.wp;
    }
    const int zb = bz * V4_ZC;
    const long long c00 = (long long)ys * sy + x0;
    auto ld = [&](const float2* a, long long c) -> DfVec4 {
        const float4* q = reinterpret_cast<const float4*>(a + c);
        const float4 u = q[0], w = q[1];
        DfVec4 d;
        d.v[0] = make_float2(u.x, u.y);
        d.v[1] = make_float2(u.z, u.w);
        d.v[2] = make_float2(w.x, w.y);
        d.v[3] = make_float2(w.z, w.w);
        return d;
    };
    DfVec4 zero;
#pragma unroll
    for (int e = 0; e < 4; ++e) zero.v[e] = make_float2(0.f, 0.f);
    auto zrow = [&](int zz) -> DfVec4 {
        if (zz < 0) return g.per[0] ? ld(p, c00 + (long long)(nz - 1) * sz) : zero;
        if (zz >= nz) return g.per[0] ? ld(p, c00) : zero;
        return ld(p, c00 + (long long)zz * sz);
    };
    DfVec4 zm = zrow(zb - 1), zc = zrow(zb);
#pragma unroll
    for (int k = 0; k < V4_ZC; ++k) {
        const int zz = zb + k;
        const DfVec4 zp = zrow(zz + 1);
        const long long c = c00 + (long long)zz * sz;
        const DfVec4 ym = nyb.wm ? ld(p, c + nyb.om) : zero;
        const DfVec4 yp = nyb.wp ? ld(p, c + nyb.op) : zero;
        const DfVec4 bv = ld(b, c);
        const float lx = __shfl_up_sync(0xffffffffu, zc.v[3].x, 1), ly = __shfl_up_sync(0xffffffffu, zc.v[3].y, 1);
        const float rx = __shfl_down_sync(0xffffffffu, zc.v[0].x, 1), ry = __shfl_down_sync(0xffffffffu, zc.v[0].y, 1);
        const float2 left = ownl ? mg_ldw_df(p, c + ol, wl) : make_float2(lx, ly);
        const float2 right = ownr ? mg_ldw_df(p, c + orr, wr) : make_float2(rx, ry);
        const int dzw = (int)(zz > 0 || g.per[0]) + (int)(zz < nz - 1 || g.per[0]);
        float rv[4], yv[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int dg = dgx[e] + dzw;
            const float2 nb[6] = {e == 0 ? left : zc.v[e - 1], e == 3 ? right : zc.v[e + 1], ym.v[e], yp.v[e],
                                  zm.v[e], zp.v[e]};
            const float r = df_resid(bv.v[e], zc.v[e], (float)dg, nb);
            rv[e] = r;
            yv[e] = mg_jacobi_from_zero(r, omega, mg_idiag<float>(g, dg));
            if (act) {
                const float rs = __fmul_rn(r, scale);
                s = __fmaf_rn(rs, rs, s);
            }
        }
        if (act) {
            *reinterpret_cast<float4*>(r32 + c) = make_float4(rv[0], rv[1], rv[2], rv[3]);
            *reinterpret_cast<float4*>(y32 + c) = make_float4(yv[0], yv[1], yv[2], yv[3]);
        }
        zm = zc;
        zc = zp;
    }
    block_partial_f(s, sc[SC_INVSCALE2], partial, bz);
    // sum(r^2) into sc[SC_RR] (k_mg_final's work)
    if (fin.ticket) {
        const unsigned int nblk = gridDim.x * gridDim.y * (gridDim.z / (BAT ? bat.nrun : 1));
        if (mg_last_block(fin.ticket, nblk)) {
            const double2 t = mg_block_total2(partial, nullptr, (int)nblk);
            if (threadIdx.x == 0 && threadIdx.y == 0) fin.sc[SC_RR] = t.x;
        }
    }
}

// ---------------------------------------------------------------- Krylov acceleration
// Mixed precision with mg_krylov: flexible conjugate gradients FCG(1) on the level-0
// equation, preconditioned by the FP32 V-cycle (zero initial guess), with the float-pair
// solution x and the float-pair true residual of iterative refinement:
//   r = b - A x (k_mg_resid_df; stop test), z = V(r), p = z + beta p with
//   beta = -(z.q)/(p.q) of the previous direction (0 on the first iteration),
//   q = A p, alpha = (p.r)/(p.q), x += alpha p.
// A x = sum(x_nb) - diag*x is the operator whose residual k_mg_resid_df forms; it is
// negative definite, which leaves alpha and beta unchanged against the positive form.
// The V-cycle is not symmetric (the restriction is not the transposed prolongation),
// hence the flexible beta. Scalars live in the solve's slots: SC_ZQ, SC_PQ, SC_PR as
// doubles, beta as a float and alpha as a float pair (so that the elementwise kernels
// do no FP64 work).


// sums of the partials of z.q and of z, then beta = -(z.q)/(p.q) of the previous
// iteration (0 on the first: k = iteration of this solve, or sc[SC_NITE] when k < 0),
// stored as a float, and the mean of z (float)
__global__ void k_fcg_final_beta(const double* __restrict__ pzq, const double* __restrict__ pz, int n, double vol,
                                 double* __restrict__ sc, int k) {
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        a += pzq[i];
        b += pz[i];
    }
    __shared__ double sm[2][32];
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) {
        sm[0][threadIdx.x >> 5] = a;
        sm[1][threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool in = threadIdx.x < (blockDim.x >> 5);
        double zq = in ? sm[0][threadIdx.x] : 0.0, zs = in ? sm[1][threadIdx.x] : 0.0;
        zq = warp_sum(zq);
        zs = warp_sum(zs);
        if (threadIdx.x == 0) fcg_set_beta(zq, zs, vol, sc, k);
    }
}

// New direction and its image, in place: p = (z - mean z) + beta p and
// q = A p = A z + beta q (A is linear and A 1 = 0, so only z is read at the
// neighbours), with the partial sums of p.q and p.r. A z = sum(z_nb) - diag*z.
// Walls and periodic directions leave A the constant null space: a right-hand side with
// a component along it (the reference's viscosity moves wall-face velocities) makes the
// stationary iteration stall at a residual floor, and would make the directions drift
// along the constant without the mean removal.
__global__ void __launch_bounds__(MG_BX * MG_BY) k_fcg_direction(const MgGeom g, const float* __restrict__ z,
                                                                 const float* __restrict__ r, float* __restrict__ p,
                                                                 float* __restrict__ q, const double* __restrict__ sc,
                                                                 double* __restrict__ ppq, double* __restrict__ ppr) {
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const float beta = reinterpret_cast<const float*>(sc + SC_BETA)[0];
    const float zmean = reinterpret_cast<const float*>(sc + SC_ZMEAN)[0];
    float spq = 0.f, spr = 0.f;
    if (x < g.n[2] && y < g.n[1]) {
        const int nz = g.n[0], z0 = blockIdx.z * MG_ZC;
        const long long sy = g.n[2], sz = (long long)g.n[1] * g.n[2];
        const MgNb nx = mg_nb(x, g.n[2], g.per[2], 1), ny = mg_nb(y, g.n[1], g.per[1], sy);
        const int dxy = (int)nx.wm + (int)nx.wp + (int)ny.wm + (int)ny.wp;
        const long long c0 = mg_at(g, z0, y, x);
        auto cell = [&](long long c, float zm, float z0v, float zp, int dg) {
            const float s = ((((mg_ldw(z, c + nx.om, nx.wm) + mg_ldw(z, c + nx.op, nx.wp)) +
                               mg_ldw(z, c + ny.om, ny.wm)) + mg_ldw(z, c + ny.op, ny.wp)) + zm) + zp;
            const float az = __fmaf_rn(-(float)dg, z0v, s);
            const float pv = __fmaf_rn(beta, p[c], __fsub_rn(z0v, zmean));
            const float qv = __fmaf_rn(beta, q[c], az);
            p[c] = pv;
            q[c] = qv;
            spq = __fmaf_rn(pv, qv, spq);
            spr = __fmaf_rn(pv, r[c], spr);
        };
        if (z0 + MG_ZC <= nz) {
            const MgNb lo = mg_nb(z0, nz, g.per[0], sz), hi = mg_nb(z0 + MG_ZC - 1, nz, g.per[0], sz);
            float col[MG_ZC + 2];
            col[0] = mg_ldw(z, c0 + lo.om, lo.wm);
#pragma unroll
            for (int k = 1; k <= MG_ZC; ++k) col[k] = z[c0 + (k - 1) * sz];
            col[MG_ZC + 1] = mg_ldw(z, c0 + (MG_ZC - 1) * sz + hi.op, hi.wp);
#pragma unroll
            for (int k = 0; k < MG_ZC; ++k)
                cell(c0 + k * sz, col[k], col[k + 1], col[k + 2],
                     dxy + (k == 0 ? 1 + (int)lo.wm : (k == MG_ZC - 1 ? 1 + (int)hi.wp : 2)));
        } else {
            for (int zz = z0; zz < nz; ++zz) {
                const long long c = c0 + (zz - z0) * sz;
                const MgNb nzb = mg_nb(zz, nz, g.per[0], sz);
                cell(c, mg_ldw(z, c + nzb.om, nzb.wm), z[c], mg_ldw(z, c + nzb.op, nzb.wp),
                     dxy + (int)nzb.wm + (int)nzb.wp);
            }
        }
    }
    block_partial2_f(spq, spr, ppq, ppr, blockIdx.z);
}

// The same with 4 consecutive x cells per thread (16-byte loads and stores: the kernel
// is bound by the latency of its loads) and z-chunks of V4_ZC cells; needs nx and nz
// divisible by 4 and V4_ZC. The x neighbours of a vector come from the adjacent lanes
// of the warp (one warp = one row segment of 128 cells), and are loaded at the warp's
// ends and at the level's x faces (periodic image or dry). Same per-cell arithmetic as
// k_fcg_direction.
__global__ void __launch_bounds__(MG_BX * MG_BY, 5) k_fcg_direction_v4(const MgGeom g, const float* __restrict__ z,
                                                                    const float* __restrict__ r, float* __restrict__ p,
                                                                    float* __restrict__ q,
                                                                    const double* __restrict__ sc,
                                                                    double* __restrict__ ppq, double* __restrict__ ppr,
                                                                    const MgFin fin = MgFin()) {
    const int nx = g.n[2], ny = g.n[1], nz = g.n[0];
    const int nx4 = nx >> 2;
    const int lane = threadIdx.x;
    const int xv = blockIdx.x * MG_BX + lane;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const float beta = reinterpret_cast<const float*>(sc + SC_BETA)[0];
    const float zmean = reinterpret_cast<const float*>(sc + SC_ZMEAN)[0];
    float spq = 0.f, spr = 0.f;
    // idle lanes shadow the last vector of the row so that every lane takes part in the
    // shuffles; only active lanes store and sum
    const bool act = xv < nx4 && y < ny;
    const int x0 = min(xv, nx4 - 1) * 4, ys = min(y, ny - 1);
    const long long sy = nx, sz = (long long)ny * nx;
    const MgNb nyb = mg_nb(ys, ny, g.per[1], sy);
    // cells x0-1 and x0+4: offsets from cell x0 and wet flags
    const bool wl = x0 > 0 || g.per[2], wr = x0 + 4 < nx || g.per[2];
    const long long ol = x0 > 0 ? -1 : (g.per[2] ? (long long)(nx - 1) : 0);
    const long long orr = x0 + 4 < nx ? 4 : (g.per[2] ? (long long)(4 - nx) : 0);
    const bool ownl = lane == 0 || x0 == 0, ownr = lane == MG_BX - 1 || x0 + 4 >= nx;
    // wet x neighbours of the four cells
    int dgx[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int xx = x0 + e;
        dgx[e] = (int)(xx > 0 || g.per[2]) + (int)(xx < nx - 1 || g.per[2]) + (int)nyb.wm + (int)nyb.wp;
    }
    const int zb = blockIdx.z * V4_ZC;
    const long long c00 = (long long)ys * sy + x0;
    auto ld4 = [&](long long c) { return *reinterpret_cast<const float4*>(z + c); };
    auto zrow = [&](int zz) -> float4 {   // z value of the vector at level row zz (periodic image or dry)
        const MgNb nzb = mg_nb(zz < 0 ? 0 : (zz >= nz ? nz - 1 : zz), nz, g.per[0], sz);
        if (zz < 0) return nzb.wm ? ld4(c00 + (long long)(nz - 1) * sz) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (zz >= nz) return nzb.wp ? ld4(c00) : make_float4(0.f, 0.f, 0.f, 0.f);
        return ld4(c00 + (long long)zz * sz);
    };
    float4 zm = zrow(zb - 1), zc = zrow(zb);
#pragma unroll
    for (int k = 0; k < V4_ZC; ++k) {
        const int zz = zb + k;
        const float4 zp = zrow(zz + 1);
        const long long c = c00 + (long long)zz * sz;
        const float4 ym = nyb.wm ? ld4(c + nyb.om) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 yp = nyb.wp ? ld4(c + nyb.op) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 pv0 = *reinterpret_cast<const float4*>(p + c);
        const float4 qv0 = *reinterpret_cast<const float4*>(q + c);
        const float4 rv = *reinterpret_cast<const float4*>(r + c);
        const float sl = __shfl_up_sync(0xffffffffu, zc.w, 1);
        const float sr = __shfl_down_sync(0xffffffffu, zc.x, 1);
        const float left = ownl ? mg_ldw(z, c + ol, wl) : sl;
        const float right = ownr ? mg_ldw(z, c + orr, wr) : sr;
        const int dzw = (int)(zz > 0 || g.per[0]) + (int)(zz < nz - 1 || g.per[0]);
        const float zv[4] = {zc.x, zc.y, zc.z, zc.w};
        const float xm[4] = {left, zc.x, zc.y, zc.z}, xp[4] = {zc.y, zc.z, zc.w, right};
        const float yv[2][4] = {{ym.x, ym.y, ym.z, ym.w}, {yp.x, yp.y, yp.z, yp.w}};
        const float zmv[4] = {zm.x, zm.y, zm.z, zm.w}, zpv[4] = {zp.x, zp.y, zp.z, zp.w};
        const float p0[4] = {pv0.x, pv0.y, pv0.z, pv0.w}, q0[4] = {qv0.x, qv0.y, qv0.z, qv0.w};
        const float rr[4] = {rv.x, rv.y, rv.z, rv.w};
        float po[4], qo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float s = ((((xm[e] + xp[e]) + yv[0][e]) + yv[1][e]) + zmv[e]) + zpv[e];
            const float az = __fmaf_rn(-(float)(dgx[e] + dzw), zv[e], s);
            po[e] = __fmaf_rn(beta, p0[e], __fsub_rn(zv[e], zmean));
            qo[e] = __fmaf_rn(beta, q0[e], az);
            if (act) {
                spq = __fmaf_rn(po[e], qo[e], spq);
                spr = __fmaf_rn(po[e], rr[e], spr);
            }
        }
        if (act) {
            *reinterpret_cast<float4*>(p + c) = make_float4(po[0], po[1], po[2], po[3]);
            *reinterpret_cast<float4*>(q + c) = make_float4(qo[0], qo[1], qo[2], qo[3]);
        }
        zm = zc;
        zc = zp;
    }
    block_partial2_f(spq, spr, ppq, ppr, blockIdx.z);
    // alpha from the totals of p.q and p.r (k_fcg_final_alpha's work)
    if (fin.ticket) {
        const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
        if (mg_last_block(fin.ticket, nblk)) {
            const double2 t = mg_block_total2(ppq, ppr, (int)nblk);
            if (threadIdx.x == 0 && threadIdx.y == 0) fcg_set_alpha(t.x, t.y, fin.sc);
        }
    }
}

// sums of p.q and p.r, then alpha = (p.r)/(p.q) stored as a float pair
__global__ void k_fcg_final_alpha(const double* __restrict__ ppq, const double* __restrict__ ppr, int n,
                                  double* __restrict__ sc) {
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        a += ppq[i];
        b += ppr[i];
    }
    __shared__ double sm[2][32];
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) {
        sm[0][threadIdx.x >> 5] = a;
        sm[1][threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool in = threadIdx.x < (blockDim.x >> 5);
        double pq = in ? sm[0][threadIdx.x] : 0.0, pr = in ? sm[1][threadIdx.x] : 0.0;
        pq = warp_sum(pq);
        pr = warp_sum(pr);
        if (threadIdx.x == 0) fcg_set_alpha(pq, pr, sc);
    }
}

// x += alpha p on the float-pair solution (level 0, elementwise)
__global__ void __launch_bounds__(256) k_fcg_xupdate(float2* __restrict__ xdf, const float* __restrict__ p,
                                                     long long n, const double* __restrict__ sc) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 alpha = reinterpret_cast<const float2*>(sc + SC_ALPHA)[0];
    xdf[i] = df_add(xdf[i], df_mul_f(p[i], alpha));
}

// Extrapolated warm start of a mixed-precision solve. The solution array x(n-1) has
// MG_HIST history arrays holding x(n-2), x(n-3), ... With `order` p and at least p + 1
// solves seen (else the highest order they allow), the start becomes the polynomial
// extrapolation of the last p + 1 solutions to the next step (equal steps; binomial
// coefficients: 2, -1; 3, -3, 1; 4, -6, 4, -1), formed in float-pair arithmetic (FP64
// here ran the kernel at a fifth of the copy bandwidth: GB300's FP64 pipe, which also
// does the float-double conversions, is a small fraction of its FP32 rate). The
// history then shifts by one. Nothing changes when the right-hand side's
// norm (scalar slot SC_NORMB, set just before) is zero or not finite: the solve then
// keeps its start (a zero right-hand side) or stops at once (blow-up).
// k_mg_hist_count, launched after, counts the solve.
constexpr int MG_HIST = 3;
struct HistPtrs {
    float2* h[MG_HIST];   // x(n-2), x(n-3), x(n-4)
};
__global__ void __launch_bounds__(256) k_mg_extrapolate(float2* __restrict__ cur, HistPtrs hp, long long n,
                                                        int order, const double* __restrict__ sc,
                                                        const int* __restrict__ count, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    cur = bshift(cur, dlt);
#pragma unroll
    for (int k = 0; k < MG_HIST; ++k) hp.h[k] = bshift(hp.h[k], dlt);
    sc = bshift(sc, dlt);
    count = bshift(count, dlt);
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double nb = sc[SC_NORMB];
    if (!(nb > 0.0 && nb <= 1.7976931348623157e308)) return;
    const int p = min(order, *count - 1);   // order the history allows
    float2 v[MG_HIST + 1];
    v[0] = cur[i];
#pragma unroll
    for (int k = 0; k < MG_HIST; ++k) v[k + 1] = (k < order) ? hp.h[k][i] : make_float2(0.f, 0.f);
    if (p >= 1) {
        float2 e;
        if (p == 1) e = df_add(make_float2(2.f * v[0].x, 2.f * v[0].y), df_neg(v[1]));
        else if (p == 2) e = df_add(df_mul_f(3.f, df_add(v[0], df_neg(v[1]))), v[2]);
        else e = df_add(df_add(df_mul_f(4.f, df_add(v[0], v[2])), df_mul_f(-6.f, v[1])), df_neg(v[3]));
        cur[i] = e;
    }
#pragma unroll
    for (int k = MG_HIST - 1; k >= 0; --k)
        if (k < order) hp.h[k][i] = v[k];
}

// one thread per run: the count of solves seen by the solution array (saturating at
// MG_HIST + 1)
__global__ void k_mg_hist_count(int* count, const double* sc, const Bat bat = Bat()) {
    const int r = threadIdx.x;
    if (bat.tab) {
        if (r >= bat.nrun || !bat.tab->active[r]) return;
        count = bshift(count, bat.tab->delta[r]);
        sc = bshift(sc, bat.tab->delta[r]);
    } else if (r > 0) {
        return;
    }
    const double nb = sc[SC_NORMB];
    if (nb > 0.0 && nb <= 1.7976931348623157e308 && *count < MG_HIST + 1) *count += 1;
}

// sum of squares of a float-pair array (high parts, squared and summed in double)
__global__ void __launch_bounds__(MG_BX * MG_BY) k_mg_sumsq_df(const MgGeom g, const float2* __restrict__ v,
                                                              double* __restrict__ partial, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    v = bshift(v, dlt);
    partial = bshift(partial, dlt);
    const int x = blockIdx.x * MG_BX + threadIdx.x;
    const int y = blockIdx.y * MG_BY + threadIdx.y;
    const int z0 = bz * MG_ZC;
    const int z1 = min(z0 + MG_ZC, g.n[0]) - 1;
    double s = 0.0;
    if (x < g.n[2] && y < g.n[1])
        for (int z = z0; z <= z1; ++z) {
            const double h = (double)v[mg_at(g, z, y, x)].x;
            s += h * h;
        }
    block_partial(s, partial, bz);
}

// scale of the float sums of squares: 2^-e with 2^e near rms(b) = sqrt(sum(b^2)/vol),
// and its inverse square (both exact powers of two)
__global__ void k_mg_scale(double* __restrict__ sc, double vol, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    sc = bshift(sc, dlt);
    const double nb = sc[SC_NORMB];
    int e = 0;
    if (nb > 0.0) frexp(sqrt(nb / vol), &e);
    e = max(-120, min(120, e));
    sc[SC_SCALE] = ldexp(1.0, -e);
    sc[SC_INVSCALE2] = ldexp(1.0, 2 * e);
}

__global__ void k_mg_final(const double* __restrict__ partial, int n, double* __restrict__ out,
                           const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    partial = bshift(partial, dlt);
    out = bshift(out, dlt);
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    __shared__ double sm[32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_sum(t);
        if (threadIdx.x == 0) *out = t;
    }
}

// ---------------------------------------------------------------- device-side stop test
// before the loop: res = sum(r^2)/sum(b^2) (0 when b = 0), continue while res >= tol
__device__ __forceinline__ bool finite_dev(double v) { return v == v && v <= 1.7976931348623157e308; }

// One thread per run (a single thread for one run): each run's stop test, its `live`
// flag in a batched launch, and the loop condition = any run still iterating.
__global__ void k_mg_ctl_begin(double* __restrict__ sc0, cudaGraphConditionalHandle h, double tol,
                               const Bat bat = Bat()) {
    const int r = threadIdx.x;
    bool go = false;
    if (r < bat.nrun && (!bat.tab || bat.tab->active[r])) {
        double* sc = bat.tab ? bshift(sc0, bat.tab->delta[r]) : sc0;
        const double normb = sc[SC_NORMB];
        const double res = normb > 0.0 ? sc[SC_RR] / normb : 0.0;
        sc[SC_RES] = res;
        sc[SC_NITE] = 0.0;
        if (!finite_dev(normb) || !finite_dev(res))   // non-finite input: no V-cycle (host: NYLES_BLOWUP)
            sc[SC_NONFINITE] = sc[SC_NONFINITE] + 1.0;
        else
            go = !(res < tol);
    }
    if (bat.tab && r < NYLES_MAX_BATCH) bat.tab->live[r] = go ? 1 : 0;
    const int any = __syncthreads_or(go ? 1 : 0);
    if (r == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// after each V-cycle: nite += 1; stop at maxite (res keeps its previous value, as
// solvers.f90:24-26 leaves the loop before recomputing it), else recompute res
__global__ void k_mg_ctl_step(double* __restrict__ sc0, cudaGraphConditionalHandle h, double tol, int maxite,
                              const Bat bat = Bat()) {
    const int r = threadIdx.x;
    bool go = false;
    if (r < bat.nrun && (!bat.tab || bat.tab->live[r])) {   // runs whose solve stopped keep their counters
        double* sc = bat.tab ? bshift(sc0, bat.tab->delta[r]) : sc0;
        const double nite = sc[SC_NITE] + 1.0;
        sc[SC_NITE] = nite;
        sc[SC_TOTAL] = sc[SC_TOTAL] + 1.0;
        if (nite >= (double)maxite) {
            if (sc[SC_RES] >= tol) sc[SC_NCONV] = sc[SC_NCONV] + 1.0;   // as mg_solve's count
        } else {
            const double normb = sc[SC_NORMB];
            const double res = normb > 0.0 ? sc[SC_RR] / normb : 0.0;
            sc[SC_RES] = res;
            if (!finite_dev(res))
                sc[SC_NONFINITE] = sc[SC_NONFINITE] + 1.0;
            else
                go = !(res < tol);
        }
        if (bat.tab) bat.tab->live[r] = go ? 1 : 0;
    }
    const int any = __syncthreads_or(go ? 1 : 0);
    if (r == 0) {
        if (bat.tab) bat.tab->loop_iterations += 1;
        cudaGraphSetConditional(h, any ? 1u : 0u);
    }
}

// ---------------------------------------------------------------- host side
static inline dim3 grid_zc(const int n[3], int zc) {
    return dim3((n[2] + MG_BX - 1) / MG_BX, (n[1] + MG_BY - 1) / MG_BY, (n[0] + zc - 1) / zc);
}
static const dim3 kBlk(MG_BX, MG_BY, 1);
// the grid of a batched launch repeats the one-run grid along z once per run
static inline dim3 bgrid(const MgImpl* mg, dim3 g) {
    if (mg->bat.tab) g.z *= mg->bat.nrun;
    return g;
}

// the 4-cell vector kernels apply to a level whose x and z extents allow them; zc = the
// z cells per thread (V4_ZC on level 0 and for the float-pair and Krylov kernels,
// lvl_zc below)
static inline bool use_v4(const MgImpl* mg, const int n[3], int zc = V4_ZC) {
    return mg->vec4 && n[2] % 4 == 0 && n[0] % zc == 0;
}
static inline dim3 grid_v4(const int n[3], int zc = V4_ZC) {
    return dim3((unsigned)((n[2] / 4 + MG_BX - 1) / MG_BX), (unsigned)((n[1] + MG_BY - 1) / MG_BY),
                (unsigned)(n[0] / zc));
}
// z cells per thread of the half-sweeps of level l: level 0 reuses each z row from
// registers over V4_ZC cells; the coarser levels are latency-bound (a few microseconds
// per launch whatever their size), where more blocks with shorter chains of dependent
// loads finish sooner
static inline int lvl_zc(const MgImpl* mg, int l) { return l == 0 ? V4_ZC : mg->czc; }
// coarse planes per thread of the restriction out of level l, fine planes per thread of
// the prolongation into level l (even)
static inline int lvl_rzc(const MgImpl* mg, int l) { return l == 0 ? MG_RZC : (mg->czc >= 4 ? MG_RZC : 1); }
static inline int lvl_pzc(const MgImpl* mg, int l) { return l == 0 ? V4_ZC : (mg->czc >= 4 ? V4_ZC : 2); }
static inline dim3 grid_v4_restrict(const MgGeom& gf, const MgGeom& gc, int rzc) {
    return dim3((unsigned)((gf.n[2] / 4 + MG_BX - 1) / MG_BX), (unsigned)((gc.n[1] + MG_BY - 1) / MG_BY),
                (unsigned)(gc.n[0] / rzc));
}
// ticket counter of the reductions folded into their kernels (MgFin), in a workspace
// slot zeroed when the workspace is bound
static inline unsigned int* fin_ticket(MgImpl* mg) {
    return reinterpret_cast<unsigned int*>(mg->ws + mg->off_ticket);
}

// the vector transfers between levels l and l + 1: exact halving in every direction,
// fine nx divisible by 4, and the z chunk of each kernel dividing its extent
static inline bool v4_restrict(const MgImpl* mg, const MgGeom& gf, const MgGeom& gc, int rzc) {
    if (!mg->vec4 || gf.n[2] % 4 != 0 || gc.n[0] % rzc != 0) return false;
    for (int k = 0; k < 3; ++k)
        if (gf.n[k] != 2 * gc.n[k]) return false;
    return true;
}
static inline bool v4_prolong(const MgImpl* mg, const MgGeom& gf, const MgGeom& gc, int pzc) {
    if (!mg->vec4 || gf.n[2] % 4 != 0 || gf.n[0] % pzc != 0) return false;
    for (int k = 0; k < 3; ++k)
        if (gf.n[k] != 2 * gc.n[k]) return false;
    return true;
}

// launches of the MODE-0 vector half-sweep and of the vector transfers with a z chunk
// chosen at run time
template <bool BAT>
static void launch_jacobi_v4_0(int zc, dim3 grd, cudaStream_t st, const MgGeom& g, const float* in, const float* b,
                               float* out, float om, const Bat& bt) {
    if (zc == 1)
        k_mg_jacobi_v4<0, BAT, 1><<<grd, kBlk, 0, st>>>(g, in, b, out, om, nullptr, nullptr, nullptr, nullptr, bt);
    else if (zc == 2)
        k_mg_jacobi_v4<0, BAT, 2><<<grd, kBlk, 0, st>>>(g, in, b, out, om, nullptr, nullptr, nullptr, nullptr, bt);
    else
        k_mg_jacobi_v4<0, BAT, 4><<<grd, kBlk, 0, st>>>(g, in, b, out, om, nullptr, nullptr, nullptr, nullptr, bt);
}
template <bool BAT>
static void launch_restrict_v4(int rzc, dim3 grd, cudaStream_t st, const MgGeom& gf, const float* xf, const float* bf,
                               const MgGeom& gc, float* bc, float* yc, float om, const Bat& bt) {
    if (rzc == 1)
        k_mg_restrict_v4<BAT, 1><<<grd, kBlk, 0, st>>>(gf, xf, bf, gc, bc, yc, om, bt);
    else
        k_mg_restrict_v4<BAT, MG_RZC><<<grd, kBlk, 0, st>>>(gf, xf, bf, gc, bc, yc, om, bt);
}
template <bool BAT>
static void launch_prolong_v4(int pzc, dim3 grd, cudaStream_t st, const MgGeom& gf, float* xf, const MgGeom& gc,
                              const float* xc, const Bat& bt) {
    if (pzc == 2)
        k_mg_prolong_v4<BAT, 2><<<grd, kBlk, 0, st>>>(gf, xf, gc, xc, bt);
    else
        k_mg_prolong_v4<BAT, V4_ZC><<<grd, kBlk, 0, st>>>(gf, xf, gc, xc, bt);
}

static inline MgGeom mgg(const MgImpl* mg, int l) {
    MgGeom g;
    for (int k = 0; k < 3; ++k) { g.n[k] = mg->lev[l].n[k]; g.per[k] = mg->per[k]; }
    // compute_diag (operators.f90:454-484): idiag = 1/diag where diag > 0, times the
    // smoother's damping omega (one multiplication less per cell and half-sweep)
    g.idiag[0] = 0.0;
    for (int k = 1; k < 8; ++k) g.idiag[k] = mg->omega / (double)k;
    // compute_Pcoef (operators.f90:423-452): Pcoef = 1/(prolongation of the coarse mask)
    for (int bits = 0; bits < 8; ++bits) {
        const int W = (3 + (bits & 1)) * (3 + ((bits >> 1) & 1)) * (3 + ((bits >> 2) & 1));
        g.pcoef[bits] = 1.0 / (double)W;
    }
    for (int k = 0; k < 8; ++k) {
        g.fidiag[k] = (float)g.idiag[k];
        g.fpcoef[k] = (float)g.pcoef[k];
    }
    return g;
}
static inline bool empty(const MgImpl* mg, int l) { return mg->lev[l].vol == 0; }

template <typename T>
static T* lvp(MgImpl* mg, int l, int var) {
    size_t off = var == 1 ? mg->lev[l].off_x : (var == 2 ? mg->lev[l].off_b : mg->lev[l].off_y);
    return reinterpret_cast<T*>(mg->ws + off);
}

void* mg_level_ptr(MgImpl* mg, int lev, int var) {
    if (!mg->ws || lev < 1 || lev > mg->nlevels) return nullptr;
    if (lev == 1 && mg->precision == NYLES_MIXED) {
        if (var == 1) return reinterpret_cast<char*>(mg_pdf(mg));
        if (var == 2) return mg->ws + mg->off_bdf;
    }
    size_t off = var == 1 ? mg->lev[lev - 1].off_x : (var == 2 ? mg->lev[lev - 1].off_b : mg->lev[lev - 1].off_y);
    return mg->ws + off;
}

float2* mg_pdf(MgImpl* mg) {
    return reinterpret_cast<float2*>(mg->ws + mg->off_pdf + (size_t)mg->cur_sol * mg->sol_bytes);
}
// the solutions before the current one (history arrays, h = 1..MG_HIST) and the
// current solution's count
static float2* mg_pdf_old(MgImpl* mg, int h) {
    return reinterpret_cast<float2*>(mg->ws + mg->off_pdf + (size_t)(h * mg->nsol + mg->cur_sol) * mg->sol_bytes);
}
static int* mg_hist_count(MgImpl* mg) { return reinterpret_cast<int*>(mg->ws + mg->off_hist) + mg->cur_sol; }

// mg_setup.f90:225-307 (create_hierarchy) for one rank. The reference leaves the loop
// only when x == 2 or y == 2; here coarsening also stops before an odd extent, so
// 3*2^n sizes terminate (the reference does not terminate on them).

int mg_init(MgImpl* mg, int nx, int ny, int nz, int topology, int precision, int nsol, int nhist) {
    if (nhist < 0 || nhist > MG_HIST) { set_error("multigrid: history depth out of range"); return NYLES_BAD_ARG; }
    if (nx < 2 || ny < 2 || nz < 1) { set_error("multigrid: grid too small"); return NYLES_BAD_ARG; }
    if (topology < 1 || topology > 6) { set_error("multigrid: bad topology"); return NYLES_BAD_ARG; }
    mg->precision = precision;
    mg->per[2] = (topology == NYLES_MG_XPERIO || topology == NYLES_MG_XYPERIO || topology == NYLES_MG_XYZPERIO);
    mg->per[1] = (topology == NYLES_MG_YPERIO || topology == NYLES_MG_XYPERIO || topology == NYLES_MG_XYZPERIO);
    mg->per[0] = (topology == NYLES_MG_ZPERIO || topology == NYLES_MG_XYZPERIO);
    const int nh = 3;
    int x = nx, y = ny, z = nz + 2 * nh;
    int L = 0;
    while (true) {
        if (L >= 32) { set_error("multigrid: too many levels"); return NYLES_UNSUPPORTED; }
        MgLevelDesc& d = mg->lev[L];
        d.n[0] = z - 2 * nh; d.n[1] = y; d.n[2] = x;
        if (d.n[0] < 0) d.n[0] = 0;
        d.vol = (long long)d.n[0] * d.n[1] * d.n[2];
        ++L;
        if (x == 2 || y == 2) break;
        if ((x % 2) || (y % 2) || x < 4 || y < 4) break;
        x /= 2; y /= 2; z = z / 2 + nh;
    }
    mg->nlevels = L;
    // An odd z extent above the coarsest level makes mgfor's prolongation write a ghost
    // layer (basicoperators.f90:194-229 steps k by 2 up to nz-nh); not supported.
    for (int l = 0; l + 1 < L; ++l)
        if (mg->lev[l].n[0] % 2) { set_error("multigrid: z extent must stay even above the coarsest level"); return NYLES_UNSUPPORTED; }
    if (mg->lev[0].n[0] < 1) { set_error("multigrid: empty grid"); return NYLES_BAD_ARG; }
    // workspace layout
    const size_t es = precision == NYLES_MIXED ? sizeof(float) : sizeof(double);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    for (int l = 0; l < L; ++l) {
        MgLevelDesc& d = mg->lev[l];
        d.off_x = take(d.vol * es);
        d.off_b = take(d.vol * es);
        d.off_y = take(d.vol * es);
    }
    if (precision == NYLES_MIXED) {
        mg->nsol = nsol < 1 ? 1 : nsol;
        mg->cur_sol = 0;
        mg->sol_bytes = (mg->lev[0].vol * sizeof(float2) + 255) & ~(size_t)255;
        mg->nhist = nhist;
        mg->extrap = 0;
        mg->off_pdf = take(mg->sol_bytes * mg->nsol * (1 + nhist));
        if (nhist) mg->off_hist = take(mg->nsol * sizeof(int));
        mg->off_bdf = take(mg->lev[0].vol * sizeof(float2));
        mg->off_fp = take(mg->lev[0].vol * sizeof(float));
        mg->off_fq = take(mg->lev[0].vol * sizeof(float));
    }
    // the coarsest levels whose arrays fit in one block's shared memory (two levels at
    // least, never level 0) run as one k_mg_bottom launch per V-cycle. In FP64 the block's
    // SM does the levels' FP64 work alone (~2 FP64 instructions per cycle): levels above
    // MG_BOTTOM_MAXVOL_FP64 cells are faster as grid launches spread over every SM.
    mg->bottom = L;
    mg->bottom_smem = 0;
    {
        size_t bytes = 0;
        for (int l = L - 1; l >= 1 && L - l <= MG_BOTTOM_MAXLEV; --l) {
            bytes += 3 * (size_t)mg->lev[l].vol * es;
            if (bytes > MG_BOTTOM_SMEM) break;
            if (precision != NYLES_MIXED && mg->lev[l].vol > MG_BOTTOM_MAXVOL_FP64) break;
            if (L - l >= 2) {
                mg->bottom = l;
                mg->bottom_smem = bytes;
            }
        }
        if (mg->bottom < L) {
            cudaError_t e = precision == NYLES_MIXED
                                ? cudaFuncSetAttribute(k_mg_bottom<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)MG_BOTTOM_SMEM)
                                : cudaFuncSetAttribute(k_mg_bottom<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)MG_BOTTOM_SMEM);
            if (e != cudaSuccess) return cuda_status(e, "multigrid coarse-level kernel attribute");
        }
    }
    // one partial per block of the largest reduction grid (the float-pair residual's)
    const dim3 g0 = grid_zc(mg->lev[0].n, MG_DFZC < MG_ZC ? MG_DFZC : MG_ZC);
    mg->npartial = (int)(g0.x * g0.y * g0.z);
    {
        const char* e = getenv("NYLES_GB300_SCALAR_KERNELS");
        mg->vec4 = !(e && e[0] == '1');
        const char* c = getenv("NYLES_GB300_COARSE_ZC");
        const int czc = c ? atoi(c) : 1;
        mg->czc = (czc == 2 || czc == 4) ? czc : 1;
    }
    mg->off_partial = take(mg->npartial * sizeof(double));
    mg->off_partial2 = take(mg->npartial * sizeof(double));
    mg->off_scalars = take(16 * sizeof(double));
    mg->off_ticket = take(64);
    mg->bytes = off;
    return NYLES_OK;
}

// smoothing of level l: half-sweeps x -> y -> x; with from_y the first one was already
// written into y by the kernel that set b from a zero solution. The last half-sweep
// runs in `last_mode` (k_mg_jacobi: 0 store, 1 add to the float-pair solution, 2 store
// and sum its dot product with the Krylov vector q).
template <typename T>
static void smooth(MgImpl* mg, int l, cudaStream_t st, int last_mode, bool from_y = false) {
    if (empty(mg, l)) return;
    MgGeom g = mgg(mg, l);
    const dim3 grd = grid_zc(g.n, MG_ZC);
    T* x = lvp<T>(mg, l, 1);
    T* b = lvp<T>(mg, l, 2);
    T* y = lvp<T>(mg, l, 3);
    const T om = T(mg->omega);
    ProfScope ps(mg->prof, 8, st);
    note_launch(from_y ? 1 : 2);
    if (mg->bat.tab) {   // batched (stationary mixed refinement): modes 0 and 1
        const Bat& bt = mg->bat;
        float2* pdf = last_mode == 1 ? mg_pdf(mg) : nullptr;
        if constexpr (sizeof(T) == sizeof(float)) {
            const int zc = last_mode == 1 ? V4_ZC : lvl_zc(mg, l);
            if (use_v4(mg, g.n, zc)) {
                const dim3 gv = bgrid(mg, grid_v4(g.n, zc));
                if (!from_y) launch_jacobi_v4_0<true>(zc, gv, st, g, x, b, y, om, bt);
                if (last_mode == 1)
                    k_mg_jacobi_v4<1, true><<<gv, kBlk, 0, st>>>(g, y, b, x, om, pdf, nullptr, nullptr, nullptr, bt);
                else
                    launch_jacobi_v4_0<true>(zc, gv, st, g, y, b, x, om, bt);
                return;
            }
        }
        const dim3 gb = bgrid(mg, grd);
        if (!from_y) k_mg_jacobi<T, 0, true><<<gb, kBlk, 0, st>>>(g, x, b, y, om, nullptr, nullptr, nullptr, nullptr, bt);
        if (last_mode == 1)
            k_mg_jacobi<T, 1, true><<<gb, kBlk, 0, st>>>(g, y, b, x, om, pdf, nullptr, nullptr, nullptr, bt);
        else
            k_mg_jacobi<T, 0, true><<<gb, kBlk, 0, st>>>(g, y, b, x, om, nullptr, nullptr, nullptr, nullptr, bt);
        return;
    }
    if constexpr (sizeof(T) == sizeof(float)) {
        const int zc = last_mode != 0 ? V4_ZC : lvl_zc(mg, l);
        if (use_v4(mg, g.n, zc)) {
            const dim3 gv = grid_v4(g.n, zc);
            if (!from_y) launch_jacobi_v4_0<false>(zc, gv, st, g, x, b, y, om, Bat());
            if (last_mode == 1)
                k_mg_jacobi_v4<1><<<gv, kBlk, 0, st>>>(g, y, b, x, om, mg_pdf(mg),
                                                      nullptr, nullptr, nullptr);
            else if (last_mode == 2) {   // also beta and the mean of z for the Krylov update
                MgFin fin;
                fin.ticket = fin_ticket(mg);
                fin.sc = reinterpret_cast<double*>(mg->ws + mg->off_scalars);
                fin.k = mg->fcg_k;
                fin.vol = (double)mg->lev[0].vol;
                k_mg_jacobi_v4<2><<<gv, kBlk, 0, st>>>(g, y, b, x, om, nullptr,
                                                      reinterpret_cast<const float*>(mg->ws + mg->off_fq),
                                                      reinterpret_cast<double*>(mg->ws + mg->off_partial),
                                                      reinterpret_cast<double*>(mg->ws + mg->off_partial2), Bat(),
                                                      fin);
            }
            else
                launch_jacobi_v4_0<false>(zc, gv, st, g, y, b, x, om, Bat());
            return;
        }
    }
    if (!from_y) k_mg_jacobi<T, 0><<<grd, kBlk, 0, st>>>(g, x, b, y, om, nullptr, nullptr, nullptr, nullptr);
    if (last_mode == 1)
        k_mg_jacobi<T, 1><<<grd, kBlk, 0, st>>>(g, y, b, x, om, mg_pdf(mg),
                                                nullptr, nullptr, nullptr);
    else if (last_mode == 2)
        k_mg_jacobi<T, 2><<<grd, kBlk, 0, st>>>(g, y, b, x, om, nullptr,
                                                reinterpret_cast<const T*>(mg->ws + mg->off_fq),
                                                reinterpret_cast<double*>(mg->ws + mg->off_partial),
                                                reinterpret_cast<double*>(mg->ws + mg->off_partial2));
    else
        k_mg_jacobi<T, 0><<<grd, kBlk, 0, st>>>(g, y, b, x, om, nullptr, nullptr, nullptr, nullptr);
}

// solvers.f90:35-55
// levels mg->bottom..L-1 of the V-cycle in one block (k_mg_bottom)
template <typename T>
static void bottom(MgImpl* mg, cudaStream_t st) {
    const int l0 = mg->bottom;
    if (empty(mg, l0)) return;
    MgBottom<T> a;
    a.nlev = mg->nlevels - l0;
    int off = 0;
    for (int k = 0; k < a.nlev; ++k) {
        a.g[k] = mgg(mg, l0 + k);
        a.off[k] = off;
        off += 3 * (int)mg->lev[l0 + k].vol;
    }
    a.xg = lvp<T>(mg, l0, 1);
    a.bg = lvp<T>(mg, l0, 2);
    a.omega = T(mg->omega);
    ProfScope ps(mg->prof, 8, st);
    note_launch();
    k_mg_bottom<T><<<bgrid(mg, dim3(1, 1, 1)), MgBottomThreads<T>::n, mg->bottom_smem, st>>>(a, mg->bat);
}

// level0_last: mode of the last level-0 half-sweep (see smooth)
template <typename T>
static void vcycle(MgImpl* mg, cudaStream_t st, int level0_last) {
    const int L = mg->nlevels;
    const int B = mg->bottom;   // < L: levels B..L-1 in one block
    // The first half-sweep of level 0 was written by the stop-test residual kernel that
    // precedes every V-cycle (k_mg_resid_sweep; mixed: k_mg_resid_df, from a zero
    // correction); every restricted level gets it from the restriction.
    for (int l = 0; l < L - 1 && l < B; ++l) {
        smooth<T>(mg, l, st, 0, true);
        if (!empty(mg, l + 1)) {
            MgGeom gf = mgg(mg, l), gc = mgg(mg, l + 1);
            ProfScope ps(mg->prof, 9, st);
            note_launch();
            bool done = false;
            if constexpr (sizeof(T) == sizeof(float)) {
                const int rzc = lvl_rzc(mg, l);
                if (v4_restrict(mg, gf, gc, rzc)) {
                    const dim3 gv = grid_v4_restrict(gf, gc, rzc);
                    if (mg->bat.tab)
                        launch_restrict_v4<true>(rzc, bgrid(mg, gv), st, gf, lvp<float>(mg, l, 1), lvp<float>(mg, l, 2), gc,
                                                 lvp<float>(mg, l + 1, 2), lvp<float>(mg, l + 1, 3), (float)mg->omega,
                                                 mg->bat);
                    else
                        launch_restrict_v4<false>(rzc, gv, st, gf, lvp<float>(mg, l, 1), lvp<float>(mg, l, 2), gc,
                                                  lvp<float>(mg, l + 1, 2), lvp<float>(mg, l + 1, 3), (float)mg->omega,
                                                  Bat());
                    done = true;
                }
            }
            if (!done && mg->bat.tab)
                k_mg_restrict<T, true><<<bgrid(mg, grid_zc(gc.n, MG_RZC)), kBlk, 0, st>>>(
                    gf, lvp<T>(mg, l, 1), lvp<T>(mg, l, 2), gc, lvp<T>(mg, l + 1, 2), lvp<T>(mg, l + 1, 3),
                    T(mg->omega), mg->bat);
            else if (!done)
                k_mg_restrict<T><<<grid_zc(gc.n, MG_RZC), kBlk, 0, st>>>(gf, lvp<T>(mg, l, 1), lvp<T>(mg, l, 2), gc,
                                                                        lvp<T>(mg, l + 1, 2), lvp<T>(mg, l + 1, 3),
                                                                        T(mg->omega));
        }
    }
    if (B < L)
        bottom<T>(mg, st);
    else
        smooth<T>(mg, L - 1, st, L == 1 ? level0_last : 0, true);
    for (int l = (B < L ? B - 1 : L - 2); l >= 0; --l) {
        if (!empty(mg, l + 1)) {
            MgGeom gf = mgg(mg, l), gc = mgg(mg, l + 1);
            ProfScope ps(mg->prof, 10, st);
            note_launch();
            bool done = false;
            if constexpr (sizeof(T) == sizeof(float)) {
                const int pzc = lvl_pzc(mg, l);
                if (v4_prolong(mg, gf, gc, pzc)) {
                    if (mg->bat.tab)
                        launch_prolong_v4<true>(pzc, bgrid(mg, grid_v4(gf.n, pzc)), st, gf, lvp<float>(mg, l, 1), gc,
                                                lvp<float>(mg, l + 1, 1), mg->bat);
                    else
                        launch_prolong_v4<false>(pzc, grid_v4(gf.n, pzc), st, gf, lvp<float>(mg, l, 1), gc,
                                                 lvp<float>(mg, l + 1, 1), Bat());
                    done = true;
                }
            }
            if (!done && mg->bat.tab)
                k_mg_prolong<T, true><<<bgrid(mg, grid_zc(gf.n, MG_ZC)), kBlk, 0, st>>>(
                    gf, lvp<T>(mg, l, 1), gc, lvp<T>(mg, l + 1, 1), mg->bat);
            else if (!done)
                k_mg_prolong<T><<<grid_zc(gf.n, MG_ZC), kBlk, 0, st>>>(gf, lvp<T>(mg, l, 1), gc, lvp<T>(mg, l + 1, 1));
        }
        smooth<T>(mg, l, st, l == 0 ? level0_last : 0);
    }
}

static int read_scalar(MgImpl* mg, double* host_out, cudaStream_t st) {
    double* out = reinterpret_cast<double*>(mg->ws + mg->off_scalars);
    cudaError_t e = cudaMemcpyAsync(host_out, out, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e, "multigrid norm");
}

static double* scalars(MgImpl* mg) { return reinterpret_cast<double*>(mg->ws + mg->off_scalars); }

// enqueue sum(v^2) (MODE 0) or sum(r^2) (MODE 1) of level 1 into *out
template <typename T, int MODE>
static void enqueue_sumsq(MgImpl* mg, const MgGeom& g, const T* v, const T* b, double* out, cudaStream_t st) {
    double* part = reinterpret_cast<double*>(mg->ws + mg->off_partial);
    const dim3 grd = grid_zc(g.n, MG_ZC);
    ProfScope ps(mg->prof, 11, st);
    note_launch(2);
    k_mg_sumsq<T, MODE><<<grd, kBlk, 0, st>>>(g, v, b, part);
    k_mg_final<<<1, 1024, 0, st>>>(part, (int)(grd.x * grd.y * grd.z), out);
}

// mixed precision: enqueue sum(b^2) of the float-pair right-hand side into
// sc[SC_NORMB] and the scale of the residual sums
static void enqueue_normb_df(MgImpl* mg, cudaStream_t st) {
    MgGeom g = mgg(mg, 0);
    double* part = reinterpret_cast<double*>(mg->ws + mg->off_partial);
    double* sc = reinterpret_cast<double*>(mg->ws + mg->off_scalars);
    const dim3 grd = grid_zc(g.n, MG_ZC);
    ProfScope ps(mg->prof, 11, st);
    note_launch(3);
    k_mg_sumsq_df<<<bgrid(mg, grd), kBlk, 0, st>>>(g, reinterpret_cast<const float2*>(mg->ws + mg->off_bdf), part,
                                                   mg->bat);
    k_mg_final<<<bgrid(mg, dim3(1, 1, 1)), 1024, 0, st>>>(part, (int)(grd.x * grd.y * grd.z), sc + SC_NORMB, mg->bat);
    k_mg_scale<<<bgrid(mg, dim3(1, 1, 1)), 1, 0, st>>>(sc, (double)mg->lev[0].vol, mg->bat);
}

// mixed precision: enqueue the float-pair residual (also the next correction's rhs)
// and its sum of squares into sc[SC_RR]
static void enqueue_resid_df(MgImpl* mg, cudaStream_t st) {
    MgGeom g = mgg(mg, 0);
    double* part = reinterpret_cast<double*>(mg->ws + mg->off_partial);
    double* sc = reinterpret_cast<double*>(mg->ws + mg->off_scalars);
    const bool v4 = use_v4(mg, g.n);
    const dim3 grd = v4 ? grid_v4(g.n) : grid_zc(g.n, MG_DFZC);
    ProfScope ps(mg->prof, 11, st);
    note_launch(v4 ? 1 : 2);
    const float2* pdf = mg_pdf(mg);
    const float2* bdf = reinterpret_cast<const float2*>(mg->ws + mg->off_bdf);
    MgFin fin;   // the vector kernel also adds the partials into sc[SC_RR]
    fin.ticket = fin_ticket(mg);
    fin.sc = sc;
    if (mg->bat.tab) {
        if (v4)
            k_mg_resid_df_v4<true><<<bgrid(mg, grd), kBlk, 0, st>>>(g, pdf, bdf, lvp<float>(mg, 0, 2), lvp<float>(mg, 0, 3),
                                                                    (float)mg->omega, sc, part, mg->bat, fin);
        else
            k_mg_resid_df<true><<<bgrid(mg, grd), kBlk, 0, st>>>(g, pdf, bdf, lvp<float>(mg, 0, 2), lvp<float>(mg, 0, 3),
                                                                 (float)mg->omega, sc, part, mg->bat);
    } else if (v4) {
        k_mg_resid_df_v4<<<grd, kBlk, 0, st>>>(g, pdf, bdf, lvp<float>(mg, 0, 2), lvp<float>(mg, 0, 3),
                                               (float)mg->omega, sc, part, Bat(), fin);
    } else {
        k_mg_resid_df<<<grd, kBlk, 0, st>>>(g, pdf, bdf, lvp<float>(mg, 0, 2), lvp<float>(mg, 0, 3), (float)mg->omega,
                                            sc, part);
    }
    if (!v4)
        k_mg_final<<<bgrid(mg, dim3(1, 1, 1)), 1024, 0, st>>>(part, (int)(grd.x * grd.y * grd.z), sc + SC_RR, mg->bat);
}

// FP64: enqueue the stop-test sum(r^2) into sc[SC_RR] together with the next V-cycle's
// first level-0 half-sweep (k_mg_resid_sweep)
static void enqueue_resid_sweep(MgImpl* mg, cudaStream_t st) {
    MgGeom g = mgg(mg, 0);
    double* part = reinterpret_cast<double*>(mg->ws + mg->off_partial);
    double* sc = reinterpret_cast<double*>(mg->ws + mg->off_scalars);
    const dim3 grd = grid_zc(g.n, MG_ZC);
    ProfScope ps(mg->prof, 11, st);
    note_launch(2);
    k_mg_resid_sweep<double><<<grd, kBlk, 0, st>>>(g, lvp<double>(mg, 0, 1), lvp<double>(mg, 0, 2),
                                                   lvp<double>(mg, 0, 3), mg->omega, part);
    k_mg_final<<<1, 1024, 0, st>>>(part, (int)(grd.x * grd.y * grd.z), sc + SC_RR);
}

// mixed precision with krylov: after the V-cycle left z = V(r) in level 0's x (and the
// partial sums of z.q), one FCG(1) update of the direction p and q = A p, and
// x += alpha p on the float-pair solution (k: iteration of this solve, or -1 to read it
// on the device)
static void enqueue_fcg_update(MgImpl* mg, cudaStream_t st, int k) {
    MgGeom g = mgg(mg, 0);
    double* part = reinterpret_cast<double*>(mg->ws + mg->off_partial);
    double* part2 = reinterpret_cast<double*>(mg->ws + mg->off_partial2);
    double* sc = scalars(mg);
    float* z = lvp<float>(mg, 0, 1);
    float* r = lvp<float>(mg, 0, 2);
    float* P = reinterpret_cast<float*>(mg->ws + mg->off_fp);
    float* Q = reinterpret_cast<float*>(mg->ws + mg->off_fq);
    const long long n = mg->lev[0].vol;
    const dim3 grd = grid_zc(g.n, MG_ZC);
    const int nb = (int)(grd.x * grd.y * grd.z);
    const unsigned eb = (unsigned)((n + 255) / 256);
    ProfScope ps(mg->prof, 11, st);
    if (use_v4(mg, g.n)) {
        // beta came with the V-cycle's last level-0 half-sweep (k_mg_jacobi_v4<2>); the
        // direction kernel also sets alpha
        note_launch(1);
        MgFin fin;
        fin.ticket = fin_ticket(mg);
        fin.sc = sc;
        k_fcg_direction_v4<<<grid_v4(g.n), kBlk, 0, st>>>(g, z, r, P, Q, sc, part, part2, fin);
    } else {
        // the partial sums of z.q and z were written by the V-cycle's last level-0 half-sweep
        note_launch(3);
        k_fcg_final_beta<<<1, 1024, 0, st>>>(part, part2, nb, (double)n, sc, k);
        k_fcg_direction<<<grd, kBlk, 0, st>>>(g, z, r, P, Q, sc, part, part2);
        k_fcg_final_alpha<<<1, 1024, 0, st>>>(part, part2, nb, sc);
    }
    note_launch(1);
    k_fcg_xupdate<<<eb, 256, 0, st>>>(mg_pdf(mg), P, n, sc);
}

template <typename T, int MODE>
static int sumsq(MgImpl* mg, const MgGeom& g, const T* v, const T* b, double* host_out, cudaStream_t st) {
    enqueue_sumsq<T, MODE>(mg, g, v, b, scalars(mg), st);
    return read_scalar(mg, host_out, st);
}

static int read_slot(MgImpl* mg, int slot, double* host_out, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(host_out, scalars(mg) + slot, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e, "multigrid norm");
}

// A non-finite norm means a non-finite right-hand side or solution: the solve stops
// at once with NYLES_BLOWUP (the stop rule alone would either accept it, since a NaN
// norm of b skips the iteration, or run to maxite on NaN residuals).
static bool finite_norm(double v) { return v == v && v <= 1.7976931348623157e308; }

static int blowup(MgImpl* mg, int nite, double res, const char* what) {
    mg->stats.nite = nite;
    mg->stats.res = res;
    mg->stats.solves += 1;
    mg->stats.vcycles += nite;
    mg->stats.nonfinite += 1;
    set_error(std::string("multigrid: non-finite ") + what + " (blow-up)");
    return NYLES_BLOWUP;
}

// extrapolated start of the next mixed solve (after its right-hand side norm)
static void enqueue_extrapolate(MgImpl* mg, cudaStream_t st) {
    if (!mg->extrap || mg->extrap > mg->nhist) return;
    const long long n = mg->lev[0].vol;
    const unsigned eb = (unsigned)((n + 255) / 256);
    double* sc = scalars(mg);
    note_launch(2);
    HistPtrs hp;
    for (int k = 0; k < MG_HIST; ++k) hp.h[k] = k < mg->nhist ? mg_pdf_old(mg, k + 1) : nullptr;
    k_mg_extrapolate<<<bgrid(mg, dim3(eb, 1, 1)), 256, 0, st>>>(mg_pdf(mg), hp, n, mg->extrap, sc,
                                                                 mg_hist_count(mg), mg->bat);
    k_mg_hist_count<<<1, mg->bat.tab ? NYLES_MAX_BATCH : 1, 0, st>>>(mg_hist_count(mg), sc, mg->bat);
}

// solvers.f90:8-33: stop when sum(r^2)/sum(b^2) < tol or after maxite V-cycles
int mg_solve(MgImpl* mg, cudaStream_t st) {
    if (!mg->ws) { set_error("multigrid: workspace not bound"); return NYLES_BAD_ARG; }
    MgGeom g0 = mgg(mg, 0);
    int nite = 0;
    double normb = 0.0, rr = 0.0, res = 0.0;
    int rc;
    if (mg->precision == NYLES_FP64) {
        double* b = lvp<double>(mg, 0, 2);
        if ((rc = sumsq<double, 0>(mg, g0, b, nullptr, &normb, st))) return rc;
        if (!finite_norm(normb)) return blowup(mg, 0, normb, "right-hand side");
        if (normb > 0.0) {
            enqueue_resid_sweep(mg, st);
            if ((rc = read_slot(mg, SC_RR, &rr, st))) return rc;
            res = rr / normb;
            if (!finite_norm(res)) return blowup(mg, 0, res, "residual");
        }
        while (true) {
            if (res < mg->tol) break;
            vcycle<double>(mg, st, 0);
            ++nite;
            if (nite >= mg->maxite) break;
            if (normb > 0.0) {
                enqueue_resid_sweep(mg, st);
                if ((rc = read_slot(mg, SC_RR, &rr, st))) return rc;
                res = rr / normb;
                if (!finite_norm(res)) return blowup(mg, nite, res, "residual");
            } else {
                res = 0.0;
            }
        }
    } else {
        enqueue_normb_df(mg, st);
        enqueue_extrapolate(mg, st);
        if ((rc = read_slot(mg, SC_NORMB, &normb, st))) return rc;
        if (!finite_norm(normb)) return blowup(mg, 0, normb, "right-hand side");
        if (normb > 0.0) {
            enqueue_resid_df(mg, st);
            if ((rc = read_slot(mg, SC_RR, &rr, st))) return rc;
            res = rr / normb;
            if (!finite_norm(res)) return blowup(mg, 0, res, "residual");
        }
        while (true) {
            if (res < mg->tol) break;
            if (mg->krylov) {              // z = V(r) preconditions an FCG(1) update of p
                mg->fcg_k = nite;
                vcycle<float>(mg, st, 2);
                enqueue_fcg_update(mg, st, nite);
            } else {
                vcycle<float>(mg, st, 1);   // FP32 correction of the residual equation, added to p
            }
            ++nite;
            if (nite >= mg->maxite) break;
            if (normb > 0.0) {
                enqueue_resid_df(mg, st);
                if ((rc = read_slot(mg, SC_RR, &rr, st))) return rc;
                res = rr / normb;
                if (!finite_norm(res)) return blowup(mg, nite, res, "residual");
            } else {
                res = 0.0;
            }
        }
    }
    mg->stats.nite = nite;
    mg->stats.res = res;
    mg->stats.solves += 1;
    mg->stats.vcycles += nite;
    if (res >= mg->tol && nite >= mg->maxite) mg->stats.not_converged += 1;
    return cuda_status(cudaGetLastError(), "multigrid solve");
}

// ---------------------------------------------------------------- graph mode
void GraphBuilder::begin_segment() {
    if (error) return;
    cudaError_t e = cudaStreamBeginCaptureToGraph(st, graph, deps.empty() ? nullptr : deps.data(), nullptr,
                                                  deps.size(), cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) error = cuda_status(e, "cudaStreamBeginCaptureToGraph");
}

void GraphBuilder::end_segment() {
    if (error) return;
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t* d = nullptr;
    size_t n = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &status, nullptr, nullptr, &d, nullptr, &n);
    if (e == cudaSuccess) {
        std::vector<cudaGraphNode_t> frontier(d, d + n);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(st, &g);
        if (e == cudaSuccess) deps.swap(frontier);
    }
    if (e != cudaSuccess) error = cuda_status(e, "graph segment capture");
}

// The same solve as mg_solve with the stop test on the device: norms and the first
// residual, then a while-node whose body is one V-cycle, the residual norm and the
// control kernel. Called with a segment of gb open; leaves a new segment open.
int mg_solve_graph(MgImpl* mg, GraphBuilder& gb) {
    if (!mg->ws) { set_error("multigrid: workspace not bound"); return NYLES_BAD_ARG; }
    cudaStream_t st = gb.st;
    MgGeom g0 = mgg(mg, 0);
    double* sc = scalars(mg);
    const bool mixed = mg->precision == NYLES_MIXED;
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, gb.graph, 0, 0);
    if (e != cudaSuccess) return gb.error = cuda_status(e, "cudaGraphConditionalHandleCreate");
    if (!mixed) {
        enqueue_sumsq<double, 0>(mg, g0, lvp<double>(mg, 0, 2), (const double*)nullptr, sc + SC_NORMB, st);
        enqueue_resid_sweep(mg, st);
    } else {
        enqueue_normb_df(mg, st);
        enqueue_extrapolate(mg, st);
        enqueue_resid_df(mg, st);
    }
    const unsigned nctl = mg->bat.tab ? NYLES_MAX_BATCH : 1;   // one thread per run
    k_mg_ctl_begin<<<1, nctl, 0, st>>>(sc, h, mg->tol, mg->bat);
    note_launch();
    gb.end_segment();
    if (gb.error) return gb.error;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, gb.graph, gb.deps.empty() ? nullptr : gb.deps.data(), nullptr, gb.deps.size(), &p);
    if (e != cudaSuccess) return gb.error = cuda_status(e, "cudaGraphAddNode(while)");
    cudaGraph_t body = p.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return gb.error = cuda_status(e, "capture of the multigrid loop body");
    const long long l0 = nyles_launch_count();
    const int gate0 = mg->bat.gate;
    mg->bat.gate = GATE_LIVE;   // batched: runs whose solve has stopped skip the loop body
    if (!mixed) {
        vcycle<double>(mg, st, 0);
        enqueue_resid_sweep(mg, st);
    } else if (mg->krylov) {
        mg->fcg_k = -1;
        vcycle<float>(mg, st, 2);
        enqueue_fcg_update(mg, st, -1);
        enqueue_resid_df(mg, st);
    } else {
        vcycle<float>(mg, st, 1);
        enqueue_resid_df(mg, st);
    }
    mg->bat.gate = gate0;
    k_mg_ctl_step<<<1, nctl, 0, st>>>(sc, h, mg->tol, mg->maxite, mg->bat);
    note_launch();
    gb.body_kernels = nyles_launch_count() - l0;
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess) return gb.error = cuda_status(e, "end of the multigrid loop body");
    gb.deps.assign(1, node);
    gb.begin_segment();
    return gb.error;
}

int mg_read_device_stats(MgImpl* mg, cudaStream_t st, MgDeviceStats* out) {
    double h[SC_NONFINITE + 1];
    cudaError_t e = cudaMemcpyAsync(h, scalars(mg), sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e, "multigrid statistics read-back");
    out->nite = (int)h[SC_NITE];
    out->res = h[SC_RES];
    out->vcycles = (long long)h[SC_TOTAL];
    out->not_converged = (long long)h[SC_NCONV];
    out->nonfinite = (long long)h[SC_NONFINITE];
    return NYLES_OK;
}

int mg_reset_history(MgImpl* mg) {
    if (!mg->nhist || !mg->ws) return NYLES_OK;
    return cuda_status(cudaMemset(mg->ws + mg->off_hist, 0, mg->nsol * sizeof(int)), "multigrid history reset");
}

int mg_zero_scalars(MgImpl* mg) {
    cudaError_t e = cudaMemset(scalars(mg), 0, 16 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(mg->ws + mg->off_ticket, 0, 64);
    if (e == cudaSuccess && mg->nhist) e = cudaMemset(mg->ws + mg->off_hist, 0, mg->nsol * sizeof(int));
    return cuda_status(e, "multigrid scalars reset");
}

}  // namespace nyles
