// Stencil kernels of the Nyles time step: right-hand side (tracer advection, vortex
// force, Bernoulli, viscosity), time-scheme updates, periodic halo fill, divergence,
// and the projection correction fused with the contravariant velocity, vorticity and
// kinetic energy.
//
// Every kernel walks the full model arrays, halo included, and reproduces the
// reference's array-end closures there: halo cells of b, u, vor and ke are then
// replaced by their periodic images exactly where the reference fills them, while
// tracer halos keep evolving with their own right-hand side as they do in the
// reference (core/model_les.py:98-127 never fills tracers).
#include "nyles_internal.h"
#include <mutex>
#include <string>

namespace nyles {

// ---------------------------------------------------------------- RHS building blocks
// Vortex-force flux at cell c along direction fa for the velocity component whose
// contravariant partner Uf is first averaged along `aa` (offset +1), then along fa;
// the vorticity Wf is shifted by one along fa. core/fortran_vortex_force.f90:41-83
// (direc) and :119-163 (flip) are the same 1-D operation with (fa, aa) swapped.
template <typename T>
__device__ __forceinline__ T vf_flux(const T* __restrict__ Uf, const T* __restrict__ Wf, const Geom& g,
                                     long long c, int k, int fa, int aa) {
    const int n = g.N[fa];
    const long long sf = g.stride(fa), sa = g.stride(aa);
    const long long base = c - (long long)k * sf;
    T UU1 = T(0.5) * (__ldg(Uf + c) + __ldg(Uf + c + sa));
    T UU0 = (k > 0) ? T(0.5) * (__ldg(Uf + c - sf) + __ldg(Uf + c - sf + sa)) : T(0);
    T u1 = T(0.5) * (UU0 + UU1);
    // q(k) = vort(k-1), q(0) = 0
    auto Q = [&](int kk) -> T { return kk == 0 ? T(0) : __ldg(Wf + base + (long long)(kk - 1) * sf); };
    return flux1d_at(k, n, u1, Q);
}

// Tracer flux through the face to the right of the cell at index i along d.
// core/fortran_upwind.f90:68-83
template <typename T>
__device__ __forceinline__ T tr_flux(const T* __restrict__ Uf, const T* __restrict__ q, const Geom& g,
                                     long long c, int i, int d) {
    const int n = g.N[d];
    const long long s = g.stride(d);
    const long long base = c - (long long)i * s;
    auto Q = [&](int kk) -> T { return __ldg(q + base + (long long)kk * s); };
    return flux1d_at(i, n, __ldg(Uf + c), Q);
}

// REAL(4) literal coefficients of core/interpolate.f90:18-33 and
// core/interpolate_tracer.f90 (the same values), widened
template <typename T>
struct LinK {
    static __device__ __forceinline__ T c1() { return T(-1.0f / 6.0f); }
    static __device__ __forceinline__ T c2() { return T(5.0f / 6.0f); }
    static __device__ __forceinline__ T c3() { return T(2.0f / 6.0f); }
    static __device__ __forceinline__ T e1() { return T(-1.0f / 12.0f); }
    static __device__ __forceinline__ T e2() { return T(7.0f / 12.0f); }
    static __device__ __forceinline__ T b1() { return T(2.0f / 60.0f); }
    static __device__ __forceinline__ T b2() { return T(-13.0f / 60.0f); }
    static __device__ __forceinline__ T b3() { return T(47.0f / 60.0f); }
    static __device__ __forceinline__ T b4() { return T(27.0f / 60.0f); }
    static __device__ __forceinline__ T b5() { return T(-3.0f / 60.0f); }
};

template <typename T>
struct RhsArgs {
    Geom g;
    const T* b;
    const T* tr[NYLES_MAX_TR];
    const T* U[3];    // contravariant, index 0 = i (x), 1 = j (y), 2 = k (z)
    const T* W[3];    // vorticity components i, j, k
    const T* ke;
    const T* u[3];    // covariant (viscosity only)
    T* ds[NYLES_MAX_PROG];
    int ntr;
    int terms;
    int euler;        // Euler3d: no buoyancy in Bernoulli
    T half_dz;        // 0.5*dz, fortran_bernoulli.f90:49
    T vcoef[3];       // viscosity*ids2 for directions x, y, z
    T kcoef[NYLES_MAX_TR + 1][3];   // tracer diffusivity*ids2 of b, t0.. for x, y, z
    int kmask;        // bit q: diffuse tracer q (b = 0) when TERM_TRDIFF is set
    int vf_order;     // 0: WENO vortex force; 1..5: the linear branch of that order
    int lo[3], hi[3]; // k_rhs_march: index box (z, y, x) of the cells it computes
};

// every pointer of the arguments shifted by dlt bytes (batched launches)
template <typename T>
__device__ __forceinline__ void shift_rhs_args(RhsArgs<T>& a, long long dlt) {
    a.b = bshift(a.b, dlt);
    a.ke = bshift(a.ke, dlt);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        a.U[i] = bshift(a.U[i], dlt);
        a.W[i] = bshift(a.W[i], dlt);
        a.u[i] = bshift(a.u[i], dlt);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) a.ds[q] = bshift(a.ds[q], dlt);
}

// viscosity along direction d of component field u at c, core/fortran_dissipation.f90:18-33
template <typename T>
__device__ __forceinline__ T lap1d(const T* __restrict__ u, const Geom& g, long long c, int i, int d) {
    const long long s = g.stride(d);
    const int n = g.N[d];
    T fx = (i < n - 1) ? (__ldg(u + c + s) - __ldg(u + c)) : T(0);
    T fxm = (i > 0) ? (__ldg(u + c) - __ldg(u + c - s)) : T(0);
    return fx - fxm;
}

// -(flux divergence) of one tracer at a cell, accumulated direction by direction in
// the reference's order (x pass assigns, y and z passes add), core/tracer.py:59-72;
// with `diff`, each direction's diffusion k[pass]*lap follows its advection
// (core/tracer.py:74-76)
template <typename T>
__device__ __forceinline__ T tracer_rhs(const T* __restrict__ q, const T* const* U, const Geom& g, long long c,
                                        const int* pos, bool diff, T kx, T ky, T kz) {
    T acc = T(0);
    for (int pass = 0; pass < 3; ++pass) {
        const int d = 2 - pass;            // x, then y, then z
        const int i = pos[d];
        const T Fi = tr_flux(U[d], q, g, c, i, d);
        if (i > 0) {
            const T Fm = tr_flux(U[d], q, g, c - g.stride(d), i - 1, d);
            acc = (acc + Fm) - Fi;
        } else {
            acc = acc - Fi;
        }
        if (diff) acc = acc + (pass == 0 ? kx : (pass == 1 ? ky : kz)) * lap1d(q, g, c, i, d);
    }
    return acc;
}

// ---------------------------------------------------------------- linear vortex force
// The linear branch of core/fortran_vortex_force.f90 (direc :43-55, flip :121-133) with
// core/interpolate.f90:3-112, which the reference never takes (`linear = .false.` at
// :28 and :106); selected by NylesDesc.vf_order (param orderVF). Indices below are the
// Fortran ones of a line of n values: vU(i) is the vorticity at 0-based position i - 1
// (unshifted, unlike the WENO branch's q(i) = vort(i - 1)). core/interpolate.f90's top
// end differs from the tracer version: identity at i = n - 1 and n, the third-order
// stencil at n - 2.

// qp(i) (plus) or qm(i) of an odd order, 1 <= i <= n
template <typename T, typename VF>
__device__ __forceinline__ T vf_interp_odd(int i, int n, int order, bool plus, VF V) {
    using K = LinK<T>;
    if (order == 1 || i == 1 || i >= n - 1) return V(i);
    if (order == 3 || i == 2 || i == n - 2) {
        const T wa = plus ? K::c1() : K::c3(), wc = plus ? K::c3() : K::c1();
        return add_rn(add_rn(mul_rn(wa, V(i - 1)), mul_rn(K::c2(), V(i))), mul_rn(wc, V(i + 1)));
    }
    const T w0 = plus ? K::b1() : K::b5(), w1 = plus ? K::b2() : K::b4();
    const T w3 = plus ? K::b4() : K::b2(), w4 = plus ? K::b5() : K::b1();
    T v = mul_rn(w0, V(i - 2));
    v = add_rn(v, mul_rn(w1, V(i - 1)));
    v = add_rn(v, mul_rn(K::b3(), V(i)));
    v = add_rn(v, mul_rn(w3, V(i + 1)));
    return add_rn(v, mul_rn(w4, V(i + 2)));
}

// qm(i) of an even order (2: two-point mean; 4: the fourth-order centred stencil)
template <typename T, typename VF>
__device__ __forceinline__ T vf_interp_even(int i, int n, int order, VF V) {
    using K = LinK<T>;
    if (order == 2) return i == 1 ? mul_rn(T(0.5), V(1)) : mul_rn(T(0.5), add_rn(V(i - 1), V(i)));
    if (i == 1) return add_rn(mul_rn(K::e2(), V(1)), mul_rn(K::e1(), V(2)));
    if (i == 2) return add_rn(mul_rn(K::e2(), add_rn(V(1), V(2))), mul_rn(K::e1(), V(3)));
    if (i == n) return add_rn(mul_rn(K::e2(), add_rn(V(n - 1), V(n))), mul_rn(K::e1(), V(n - 2)));
    return add_rn(mul_rn(K::e2(), add_rn(V(i - 1), V(i))), mul_rn(K::e1(), add_rn(V(i - 2), V(i + 1))));
}

// The two products the reference subtracts (direc) or adds (flip) one after the other at
// 0-based position k along fa: qp(k) up(k+1) and qm(k+1) um(k+1) in Fortran indices
// (qp(0) = 0; up, um = positive and negative parts of the velocity averaged along aa,
// then along fa, as the WENO branch); even orders give qm(k+1) and 0.
template <typename T>
struct VfTerms {
    T a, b;
};
template <typename T>
__device__ __forceinline__ VfTerms<T> vf_lin(const T* __restrict__ Uf, const T* __restrict__ Wf, const Geom& g,
                                             long long c, int k, int fa, int aa, int order) {
    const int n = g.N[fa];
    const long long sf = g.stride(fa);
    const long long base = c - (long long)k * sf;
    auto V = [&](int i) -> T { return __ldg(Wf + base + (long long)(i - 1) * sf); };
    if ((order & 1) == 0) return {vf_interp_even<T>(k + 1, n, order, V), T(0)};
    const long long sa = g.stride(aa);
    const T UU1 = mul_rn(T(0.5), add_rn(__ldg(Uf + c), __ldg(Uf + c + sa)));
    const T UU0 = (k > 0) ? mul_rn(T(0.5), add_rn(__ldg(Uf + c - sf), __ldg(Uf + c - sf + sa))) : T(0);
    const T u1 = mul_rn(T(0.5), add_rn(UU0, UU1));
    const T uu = fabs(u1);
    const T up = mul_rn(T(0.5), add_rn(u1, uu)), um = mul_rn(T(0.5), sub_rn(u1, uu));
    const T qp = (k == 0) ? T(0) : vf_interp_odd<T>(k, n, order, true, V);
    const T qm = vf_interp_odd<T>(k + 1, n, order, false, V);
    return {mul_rn(qp, up), mul_rn(qm, um)};
}
template <typename T>
__device__ __forceinline__ T vf_sub(T acc, VfTerms<T> r) { return sub_rn(sub_rn(acc, r.a), r.b); }
template <typename T>
__device__ __forceinline__ T vf_add(T acc, VfTerms<T> r) { return add_rn(add_rn(acc, r.a), r.b); }

// The six vortex-force terms of one cell in the call order of core/vortex_force.py:69-81
// (triplets "ikj", "jik", "kji": direc then flip). VF = 1: WENO; VF = 2: the linear
// branch of order a.vf_order.
template <typename T, int VF>
__device__ __forceinline__ void vortex_force_cell(const RhsArgs<T>& a, long long c, int z, int y, int x, T& dux,
                                                  T& duy, T& duz) {
    const Geom& g = a.g;
    const int Nz = g.N[0], Ny = g.N[1], Nx = g.N[2];
    if (VF == 1) {
        if (y < Ny - 1) duy = duy - vf_flux(a.U[0], a.W[2], g, c, x, 2, 1);   // u_j -= U^i w_k, along i
        if (x < Nx - 1) dux = dux + vf_flux(a.U[1], a.W[2], g, c, y, 1, 2);   // u_i += U^j w_k, along j
        if (z < Nz - 1) duz = duz - vf_flux(a.U[1], a.W[0], g, c, y, 1, 0);   // u_k -= U^j w_i, along j
        if (y < Ny - 1) duy = duy + vf_flux(a.U[2], a.W[0], g, c, z, 0, 1);   // u_j += U^k w_i, along k
        if (x < Nx - 1) dux = dux - vf_flux(a.U[2], a.W[1], g, c, z, 0, 2);   // u_i -= U^k w_j, along k
        if (z < Nz - 1) duz = duz + vf_flux(a.U[0], a.W[1], g, c, x, 2, 0);   // u_k += U^i w_j, along i
    } else {
        const int o = a.vf_order;
        if (y < Ny - 1) duy = vf_sub(duy, vf_lin(a.U[0], a.W[2], g, c, x, 2, 1, o));
        if (x < Nx - 1) dux = vf_add(dux, vf_lin(a.U[1], a.W[2], g, c, y, 1, 2, o));
        if (z < Nz - 1) duz = vf_sub(duz, vf_lin(a.U[1], a.W[0], g, c, y, 1, 0, o));
        if (y < Ny - 1) duy = vf_add(duy, vf_lin(a.U[2], a.W[0], g, c, z, 0, 1, o));
        if (x < Nx - 1) dux = vf_sub(dux, vf_lin(a.U[2], a.W[1], g, c, z, 0, 2, o));
        if (z < Nz - 1) duz = vf_add(duz, vf_lin(a.U[0], a.W[1], g, c, x, 2, 0, o));
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_rhs(const RhsArgs<T> a) {
    const Geom& g = a.g;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= g.N[2] || y >= g.N[1] || z >= g.N[0]) return;
    const long long c = g.at(z, y, x);
    const int pos[3] = {z, y, x};
    const bool acc = (a.terms & TERM_ACCUMULATE) != 0;

    // ---- tracers: b first, then t0.. (core/tracer.py:59-72)
    if (a.terms & TERM_TRACER) {
        const T* Uxyz[3] = {a.U[2], a.U[1], a.U[0]};   // indexed by geometry axis z, y, x
        for (int t = 0; t <= a.ntr; ++t) {
            const T* q = (t == 0) ? a.b : a.tr[t - 1];
            const int slot = (t == 0) ? 0 : 3 + t;
            const bool diff = (a.terms & TERM_TRDIFF) && ((a.kmask >> t) & 1);
            T v = tracer_rhs(q, Uxyz, g, c, pos, diff, a.kcoef[t][0], a.kcoef[t][1], a.kcoef[t][2]);
            if (a.ds[slot]) a.ds[slot][c] = acc ? a.ds[slot][c] + v : v;
        }
    } else if (!acc) {
        for (int t = 0; t <= a.ntr; ++t) {
            const int slot = (t == 0) ? 0 : 3 + t;
            if (a.ds[slot]) a.ds[slot][c] = T(0);
        }
    }

    // ---- velocity
    if (!(a.terms & (TERM_VF | TERM_BERNOULLI | TERM_VISC)) && acc) return;
    T dux = acc ? a.ds[1][c] : T(0);
    T duy = acc ? a.ds[2][c] : T(0);
    T duz = acc ? a.ds[3][c] : T(0);
    const int Nz = g.N[0], Ny = g.N[1], Nx = g.N[2];
    if (a.terms & TERM_VF) {
        if (a.vf_order) vortex_force_cell<T, 2>(a, c, z, y, x, dux, duy, duz);
        else vortex_force_cell<T, 1>(a, c, z, y, x, dux, duy, duz);
    }
    if (a.terms & TERM_BERNOULLI) {   // core/bernoulli.py:14-23
        const T* ke = a.ke;
        if (x < Nx - 1) dux = sub_rn(dux, sub_rn(__ldg(ke + c + 1), __ldg(ke + c)));
        if (y < Ny - 1) duy = sub_rn(duy, sub_rn(__ldg(ke + c + g.sy), __ldg(ke + c)));
        if (z < Nz - 1) {
            duz = sub_rn(duz, sub_rn(__ldg(ke + c + g.sz), __ldg(ke + c)));
            if (!a.euler) duz = add_rn(duz, mul_rn(a.half_dz, add_rn(__ldg(a.b + c + g.sz), __ldg(a.b + c))));
        }
    }
    if (a.terms & TERM_VISC) {   // core/viscosity.py:5-9: direction outer, component inner
        for (int pass = 0; pass < 3; ++pass) {
            const int d = 2 - pass;
            const T cf = a.vcoef[pass];
            dux = dux + cf * lap1d(a.u[0], g, c, pos[d], d);
            duy = duy + cf * lap1d(a.u[1], g, c, pos[d], d);
            duz = duz + cf * lap1d(a.u[2], g, c, pos[d], d);
        }
    }
    a.ds[1][c] = dux;
    a.ds[2][c] = duy;
    a.ds[3][c] = duz;
}

// ---------------------------------------------------------------- z-marching RHS
// The full right-hand side with tracer face fluxes shared between the two cells of
// each face: along x through a warp shuffle (one warp = one x row of 32 cells), along
// y through shared memory, along z carried in a register while the thread marches up
// its column chunk. One WENO5 per direction and tracer per cell instead of two; same
// arithmetic and accumulation order as k_rhs.
constexpr int RZ_BX = 32, RZ_BY = 8, RZ_ZC = 16;

template <typename T>
struct TracerMarch {
    T fz_prev;
    // -(flux divergence) at (z, ys, xs); all threads of the block must call it
    // with `diff`, k[pass]*lap follows each direction's advection (core/tracer.py:74-76)
    __device__ __forceinline__ T step(const T* __restrict__ q, const T* const* U, const Geom& g, long long c, int z,
                                      int ys, int xs, T (*sfy)[RZ_BX], bool diff, T kx, T ky, T kz) {
        const int tx = threadIdx.x, ty = threadIdx.y;
        const T fx = tr_flux(U[2], q, g, c, xs, 2);
        T fxm = __shfl_up_sync(0xffffffffu, fx, 1);
        if (tx == 0 && xs > 0) fxm = tr_flux(U[2], q, g, c - 1, xs - 1, 2);
        T acc = (xs > 0) ? (T(0) + fxm) - fx : T(0) - fx;
        if (diff) acc = acc + kx * lap1d(q, g, c, xs, 2);
        const T fy = tr_flux(U[1], q, g, c, ys, 1);
        sfy[ty][tx] = fy;
        __syncthreads();
        T fym = (ty > 0) ? sfy[ty - 1][tx] : T(0);
        __syncthreads();
        if (ty == 0 && ys > 0) fym = tr_flux(U[1], q, g, c - g.sy, ys - 1, 1);
        acc = (ys > 0) ? (acc + fym) - fy : acc - fy;
        if (diff) acc = acc + ky * lap1d(q, g, c, ys, 1);
        const T fz = tr_flux(U[0], q, g, c, z, 0);
        acc = (z > 0) ? (acc + fz_prev) - fz : acc - fz;
        if (diff) acc = acc + kz * lap1d(q, g, c, z, 0);
        fz_prev = fz;
        return acc;
    }
};

// TR: buoyancy advection on; VF: vortex force off (0), WENO (1) or the linear branch
// (2); BDIFF: buoyancy diffusion on (template flags, so that the default instances carry
// none of the optional terms' registers). ds[0..3] are written.
// blocks per SM asked of the register allocator: FP32 issue-bound march (more warps
// hide its load latency), FP64 bound by the FP64 pipe
template <typename T> struct RhsMinBlocks { static constexpr int n = 5; };
template <> struct RhsMinBlocks<double> { static constexpr int n = 4; };

// BAT: batched launch (bat names the runs; ds[0..3] and the fields of each run are
// shifted to its memory; a batched instance exists for the buoyancy-and-WENO form only)
template <typename T, bool TR, int VF, bool BDIFF, bool BAT = false>
__global__ void __launch_bounds__(RZ_BX * RZ_BY, RhsMinBlocks<T>::n) k_rhs_march(const RhsArgs<T> a0,
                                                                               const Bat bat = Bat()) {
    __shared__ T sfy[RZ_BY][RZ_BX];
    int bz = blockIdx.z;
    RhsArgs<T> a = a0;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        shift_rhs_args(a, dlt);
    }
    const Geom& g = a.g;
    const int x = a.lo[2] + blockIdx.x * RZ_BX + threadIdx.x;
    const int y = a.lo[1] + blockIdx.y * RZ_BY + threadIdx.y;
    const int z0 = a.lo[0] + bz * RZ_ZC;
    const int z1 = min(z0 + RZ_ZC, a.hi[0]) - 1;
    const int Nz = g.N[0], Ny = g.N[1], Nx = g.N[2];
    const bool valid = x < a.hi[2] && y < a.hi[1];
    const int xs = min(x, a.hi[2] - 1), ys = min(y, a.hi[1] - 1);   // idle lanes shadow a real cell
    const T* Uzyx[3] = {a.U[2], a.U[1], a.U[0]};
    TracerMarch<T> tm;
    tm.fz_prev = T(0);
    if (TR && z0 > 0) tm.fz_prev = tr_flux(Uzyx[0], a.b, g, g.at(z0 - 1, ys, xs), z0 - 1, 0);
    for (int z = z0; z <= z1; ++z) {
        const long long c = g.at(z, ys, xs);
        const int pos[3] = {z, ys, xs};
        T db = T(0);
        if (TR) db = tm.step(a.b, Uzyx, g, c, z, ys, xs, sfy, BDIFF, a.kcoef[0][0], a.kcoef[0][1], a.kcoef[0][2]);
        T dux = T(0), duy = T(0), duz = T(0);
        if (VF) vortex_force_cell<T, VF>(a, c, z, ys, xs, dux, duy, duz);
        {
            const T* ke = a.ke;
            if (xs < Nx - 1) dux = sub_rn(dux, sub_rn(__ldg(ke + c + 1), __ldg(ke + c)));
            if (ys < Ny - 1) duy = sub_rn(duy, sub_rn(__ldg(ke + c + g.sy), __ldg(ke + c)));
            if (z < Nz - 1) {
                duz = sub_rn(duz, sub_rn(__ldg(ke + c + g.sz), __ldg(ke + c)));
                if (!a.euler) duz = add_rn(duz, mul_rn(a.half_dz, add_rn(__ldg(a.b + c + g.sz), __ldg(a.b + c))));
            }
        }
        if (a.terms & TERM_VISC) {
            for (int pass = 0; pass < 3; ++pass) {
                const int d = 2 - pass;
                const T cf = a.vcoef[pass];
                dux = dux + cf * lap1d(a.u[0], g, c, pos[d], d);
                duy = duy + cf * lap1d(a.u[1], g, c, pos[d], d);
                duz = duz + cf * lap1d(a.u[2], g, c, pos[d], d);
            }
        }
        if (valid) {
            a.ds[0][c] = db;
            a.ds[1][c] = dux;
            a.ds[2][c] = duy;
            a.ds[3][c] = duz;
        }
    }
}

// ---------------------------------------------------------------- right-hand side, 32-bit offsets
// k_rhs_march<T, true, 1, false> (buoyancy advection, WENO vortex force, Bernoulli,
// viscosity) for arrays of fewer than 2^31 cells: the same operations in the same order
// (values equal up to where the compiler fuses multiply-adds), with fewer instructions
// per cell:
//  - 32-bit offsets; the six values around a face are loaded at offsets shared by every
//    field read along that direction (x: constant offsets from one pointer; y and z:
//    c + k sy and c + k sz formed once per cell);
//  - the upwind side is chosen among the six loaded values, so every reconstruction is
//    one weno5 on registers (no data-dependent addresses);
//  - the advecting velocity averaged at the face behind the cell, (UU0 of vf_flux),
//    comes from the neighbouring lane along x and from the previous cell of the column
//    along z instead of two more loads;
//  - within three cells of an array end, where flux1d_at takes a closure branch, the
//    reconstruction falls back to flux1d_at.

// u * weno5 of the five values upwind of the face between v[2] and v[3] (flux1d_at's
// interior branch): v[0..4] for u > 0, v[5..1] otherwise
template <typename T>
__device__ __forceinline__ T weno5_upwind(T u, const T (&v)[6]) {
    const bool pos = u > T(0);
    const T qa = pos ? v[0] : v[5];
    const T qb = pos ? v[1] : v[4];
    const T qc = pos ? v[2] : v[3];
    const T qd = pos ? v[3] : v[2];
    const T qe = pos ? v[4] : v[1];
    return u * weno5(qa, qb, qc, qd, qe);
}

// flux1d_at near an array end, out of line: the closures are rare (walls), and inlined
// at the nine reconstruction sites they would multiply the kernel's code size
template <typename T>
__device__ __noinline__ T tr_flux_closure(const T* __restrict__ q, T u, int base, int i, int n, int s) {
    auto Q = [&](int kk) -> T { return __ldg(q + base + kk * s); };
    return flux1d_at(i, n, u, Q);
}
template <typename T>
__device__ __noinline__ T vf_flux_closure(const T* __restrict__ W, T u1, int base, int i, int n, int s) {
    auto Q = [&](int kk) -> T { return kk == 0 ? T(0) : __ldg(W + base + (kk - 1) * s); };
    return flux1d_at(i, n, u1, Q);
}

// tracer flux at index i of a line through c with stride s (flux1d_at of tr_flux);
// o[k] = c + (k - 3) s
template <typename T>
__device__ __forceinline__ T tr_flux32(const T* __restrict__ q, T u, int c, int i, int n, int s, bool fast,
                                       const int (&o)[7]) {
    if (fast) {
        T v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = __ldg(q + o[k + 1]);
        return weno5_upwind(u, v);
    }
    return tr_flux_closure(q, u, c - i * s, i, n, s);
}
// the same along x (stride 1: constant offsets)
template <typename T>
__device__ __forceinline__ T tr_flux32x(const T* __restrict__ q, T u, int c, int i, int n, bool fast) {
    if (fast) {
        T v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = __ldg(q + c + (k - 2));
        return weno5_upwind(u, v);
    }
    return tr_flux_closure(q, u, c - i, i, n, 1);
}

// ---- two FP32 reconstructions at once. Blackwell issues two FP32 lanes' worth of
// multiply-adds in one paired instruction (__ffma2_rn, __fadd2_rn, __fmul2_rn), and the
// FP32 right-hand side is bound by instruction issue: the two vortex-force fluxes that
// share a direction (and so their load offsets) are reconstructed together. The same
// formula as weno5<float>; the weights' divisions stay per component (hardware
// reciprocal).
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 weno5_x2(float2 qmm, float2 qm, float2 q0, float2 qp, float2 qpp) {
    typedef WenoK<float> K;
    const float2 qi1 = __ffma2_rn(f2s(K::c116()), q0, __ffma2_rn(f2s(-K::c76()), qm, __fmul2_rn(f2s(K::c13()), qmm)));
    const float2 qi2 = __ffma2_rn(f2s(K::c13()), qp, __ffma2_rn(f2s(K::c56()), q0, __fmul2_rn(f2s(-K::c16()), qm)));
    const float2 qi3 = __ffma2_rn(f2s(-K::c16()), qpp, __ffma2_rn(f2s(K::c56()), qp, __fmul2_rn(f2s(K::c13()), q0)));
    const float2 a1 = __fadd2_rn(__ffma2_rn(f2s(-2.f), qm, qmm), q0);
    const float2 b1 = __ffma2_rn(f2s(3.f), q0, __ffma2_rn(f2s(-4.f), qm, qmm));
    const float2 a2 = __fadd2_rn(__ffma2_rn(f2s(-2.f), q0, qm), qp);
    const float2 b2 = __ffma2_rn(f2s(-1.f), qp, qm);
    const float2 a3 = __fadd2_rn(__ffma2_rn(f2s(-2.f), qp, q0), qpp);
    const float2 b3 = __fadd2_rn(__ffma2_rn(f2s(-4.f), qp, __fmul2_rn(f2s(3.f), q0)), qpp);
    auto beta = [&](float2 a, float2 b) {
        return __ffma2_rn(__fmul2_rn(f2s(K::k1()), a), a, __fmul2_rn(__fmul2_rn(f2s(0.25f), b), b));
    };
    const float2 be1 = beta(a1, b1), be2 = beta(a2, b2), be3 = beta(a3, b3);
    const float2 t = __ffma2_rn(f2s(-1.f), be3, be1);
    const float2 tau5 = make_float2(fabsf(t.x), fabsf(t.y));
    const float2 d1 = __fadd2_rn(be1, f2s(K::eps5())), d2 = __fadd2_rn(be2, f2s(K::eps5())),
                 d3 = __fadd2_rn(be3, f2s(K::eps5()));
    const float2 r1 = make_float2(__fdividef(tau5.x, d1.x), __fdividef(tau5.y, d1.y));
    const float2 r2 = make_float2(__fdividef(tau5.x, d2.x), __fdividef(tau5.y, d2.y));
    const float2 r3 = make_float2(__fdividef(tau5.x, d3.x), __fdividef(tau5.y, d3.y));
    const float2 w1 = __fadd2_rn(f2s(1.f), r1);
    const float2 w2 = __fmul2_rn(f2s(6.f), __fadd2_rn(f2s(1.f), r2));
    const float2 w3 = __fmul2_rn(f2s(3.f), __fadd2_rn(f2s(1.f), r3));
    const float2 num = __ffma2_rn(w3, qi3, __ffma2_rn(w2, qi2, __fmul2_rn(w1, qi1)));
    const float2 den = __fadd2_rn(__fadd2_rn(w1, w2), w3);
    return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
}
// u * weno5_x2 of the five values upwind of the face, each component on its own side
__device__ __forceinline__ float2 weno5_upwind_x2(float2 u, const float2 (&v)[6]) {
    const bool px = u.x > 0.f, py = u.y > 0.f;
    auto sel = [&](int a, int b) { return make_float2(px ? v[a].x : v[b].x, py ? v[a].y : v[b].y); };
    return __fmul2_rn(u, weno5_x2(sel(0, 5), sel(1, 4), sel(2, 3), sel(3, 2), sel(4, 1)));
}
// vf_flux32 of two vorticity fields along one direction (offsets o shared)
__device__ __forceinline__ float2 vf_flux32_x2(const float* __restrict__ Wa, const float* __restrict__ Wb, float2 u1,
                                               int c, int i, int n, int s, bool fast, const int (&o)[7]) {
    if (fast) {
        float2 v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = make_float2(__ldg(Wa + o[k]), __ldg(Wb + o[k]));
        return weno5_upwind_x2(u1, v);
    }
    return make_float2(vf_flux_closure(Wa, u1.x, c - i * s, i, n, s), vf_flux_closure(Wb, u1.y, c - i * s, i, n, s));
}
__device__ __forceinline__ float2 vf_flux32x_x2(const float* __restrict__ Wa, const float* __restrict__ Wb, float2 u1,
                                                int c, int i, int n, bool fast) {
    if (fast) {
        float2 v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = make_float2(__ldg(Wa + c + (k - 3)), __ldg(Wb + c + (k - 3)));
        return weno5_upwind_x2(u1, v);
    }
    return make_float2(vf_flux_closure(Wa, u1.x, c - i, i, n, 1), vf_flux_closure(Wb, u1.y, c - i, i, n, 1));
}

// vortex-force reconstruction of vf_flux given u1: q(kk) = W(kk - 1), q(0) = 0
template <typename T>
__device__ __forceinline__ T vf_flux32(const T* __restrict__ W, T u1, int c, int i, int n, int s, bool fast,
                                       const int (&o)[7]) {
    if (fast) {
        T v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = __ldg(W + o[k]);
        return weno5_upwind(u1, v);
    }
    return vf_flux_closure(W, u1, c - i * s, i, n, s);
}
template <typename T>
__device__ __forceinline__ T vf_flux32x(const T* __restrict__ W, T u1, int c, int i, int n, bool fast) {
    if (fast) {
        T v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = __ldg(W + c + (k - 3));
        return weno5_upwind(u1, v);
    }
    return vf_flux_closure(W, u1, c - i, i, n, 1);
}

// blocks per SM asked of the register allocator: 48 registers (the closure branches out
// of line; inlined, they took it to 64). The paired reconstructions spill a few values
// at 48 and still beat 4 blocks per SM at 64 registers (2.28 vs 2.41 ms per 256^3 step)
template <typename T> struct LesMinBlocks { static constexpr int n = 5; };

template <typename T, bool BAT>
__global__ void __launch_bounds__(RZ_BX * RZ_BY, LesMinBlocks<T>::n) k_rhs_les(const RhsArgs<T> a0,
                                                                             const Bat bat = Bat()) {
    __shared__ T sfy[RZ_BY][RZ_BX];
    int bz = blockIdx.z;
    RhsArgs<T> a = a0;
    if constexpr (BAT) {
        long long dlt;
        if (!batch_enter(bat, bz, dlt)) return;
        shift_rhs_args(a, dlt);
    }
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = a.lo[2] + blockIdx.x * RZ_BX + tx;
    const int y = a.lo[1] + blockIdx.y * RZ_BY + ty;
    const int z0 = a.lo[0] + bz * RZ_ZC;
    const int z1 = min(z0 + RZ_ZC, a.hi[0]) - 1;
    const int Nz = a.g.N[0], Ny = a.g.N[1], Nx = a.g.N[2];
    const int sy = (int)a.g.sy, sz = (int)a.g.sz;
    const bool valid = x < a.hi[2] && y < a.hi[1];
    const int xs = min(x, a.hi[2] - 1), ys = min(y, a.hi[1] - 1);   // idle lanes shadow a real cell
    const T* __restrict__ b = a.b;
    const T* __restrict__ U0 = a.U[0];
    const T* __restrict__ U1 = a.U[1];
    const T* __restrict__ U2 = a.U[2];
    const T* __restrict__ W0 = a.W[0];
    const T* __restrict__ W1 = a.W[1];
    const T* __restrict__ W2 = a.W[2];
    const T* __restrict__ ke = a.ke;
    // interior reconstructions: tracer 2 <= i <= n - 4, vortex force 3 <= i <= n - 4
    const bool xt = xs >= 2 && xs <= Nx - 4, xv = xs >= 3 && xs <= Nx - 4;
    const bool yt = ys >= 2 && ys <= Ny - 4, yv = ys >= 3 && ys <= Ny - 4;
    const bool ylo = ys < Ny - 1, xlo = xs < Nx - 1;
    const int cxy = ys * sy + xs;
    // carried up the column: the tracer flux through the face below the cell and the
    // two z-fluxes' velocities averaged at that face
    T fz_prev = T(0), uu_zy = T(0), uu_zx = T(0);
    if (z0 > 0) {
        const int c = (z0 - 1) * sz + cxy;
        int oz[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) oz[k] = c + (k - 3) * sz;
        const int zm = z0 - 1;
        fz_prev = tr_flux32(b, __ldg(U2 + c), c, zm, Nz, sz, zm >= 2 && zm <= Nz - 4, oz);
        if (ylo) uu_zy = T(0.5) * (__ldg(U2 + c) + __ldg(U2 + c + sy));
        if (xlo) uu_zx = T(0.5) * (__ldg(U2 + c) + __ldg(U2 + c + 1));
    }
    for (int z = z0; z <= z1; ++z) {
        const int c = z * sz + cxy;
        const bool zt = z >= 2 && z <= Nz - 4, zv = z >= 3 && z <= Nz - 4;
        const bool zlo = z < Nz - 1;
        // The fluxes are formed direction by direction (z, y, x: one set of offsets
        // live at a time) and summed afterwards in the order of TracerMarch::step and
        // vortex_force_cell.
        T fz, f4 = T(0), f5 = T(0);
        {
            int oz[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) oz[k] = c + (k - 3) * sz;
            fz = tr_flux32(b, __ldg(U2 + c), c, z, Nz, sz, zt, oz);
            // f4 (ylo): u_j += U^k w_i along k (U^k averaged along j); f5 (xlo): u_i -= U^k
            // w_j along k (U^k averaged along i); reconstructed as a pair
            float2 u45 = make_float2(0.f, 0.f);
            if (ylo) {
                const T uu1 = T(0.5) * (__ldg(U2 + c) + __ldg(U2 + c + sy));
                const T uu0 = z > 0 ? uu_zy : T(0);
                uu_zy = uu1;
                u45.x = T(0.5) * (uu0 + uu1);
            }
            if (xlo) {
                const T uu1 = T(0.5) * (__ldg(U2 + c) + __ldg(U2 + c + 1));
                const T uu0 = z > 0 ? uu_zx : T(0);
                uu_zx = uu1;
                u45.y = T(0.5) * (uu0 + uu1);
            }
            if (ylo || xlo) {
                const float2 f45 = vf_flux32_x2(W0, W1, u45, c, z, Nz, sz, zv, oz);
                f4 = f45.x;
                f5 = f45.y;
            }
        }
        T fy, fym, f2 = T(0), f3 = T(0);
        {
            int oy[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) oy[k] = c + (k - 3) * sy;
            fy = tr_flux32(b, __ldg(U1 + c), c, ys, Ny, sy, yt, oy);
            sfy[ty][tx] = fy;
            __syncthreads();
            fym = (ty > 0) ? sfy[ty - 1][tx] : T(0);
            __syncthreads();
            // f2 (xlo): u_i += U^j w_k along j (U^j averaged along i); f3 (zlo): u_k -= U^j
            // w_i along j (U^j averaged along k)
            float2 u23 = make_float2(0.f, 0.f);
            if (xlo) {
                const T uu1 = T(0.5) * (__ldg(U1 + c) + __ldg(U1 + c + 1));
                const T uu0 = ys > 0 ? T(0.5) * (__ldg(U1 + c - sy) + __ldg(U1 + c - sy + 1)) : T(0);
                u23.x = T(0.5) * (uu0 + uu1);
            }
            if (zlo) {
                const T uu1 = T(0.5) * (__ldg(U1 + c) + __ldg(U1 + c + sz));
                const T uu0 = ys > 0 ? T(0.5) * (__ldg(U1 + c - sy) + __ldg(U1 + c - sy + sz)) : T(0);
                u23.y = T(0.5) * (uu0 + uu1);
            }
            if (xlo || zlo) {
                const float2 f23 = vf_flux32_x2(W2, W0, u23, c, ys, Ny, sy, yv, oy);
                f2 = f23.x;
                f3 = f23.y;
            }
        }
        if (ty == 0 && ys > 0) {   // the face below the block's first row
            const int cm = c - sy;
            int om[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) om[k] = cm + (k - 3) * sy;
            fym = tr_flux32(b, __ldg(U1 + cm), cm, ys - 1, Ny, sy, ys - 1 >= 2 && ys - 1 <= Ny - 4, om);
        }
        T fx, fxm, f1 = T(0), f6 = T(0);
        {
            fx = tr_flux32x(b, __ldg(U0 + c), c, xs, Nx, xt);
            fxm = __shfl_up_sync(0xffffffffu, fx, 1);
            if (tx == 0 && xs > 0) fxm = tr_flux32x(b, __ldg(U0 + c - 1), c - 1, xs - 1, Nx,
                                                     xs - 1 >= 2 && xs - 1 <= Nx - 4);
            // f1 (ylo): u_j -= U^i w_k along i (U^i averaged along j); f6 (zlo): u_k += U^i
            // w_j along i (U^i averaged along k)
            float2 u16 = make_float2(0.f, 0.f);
            if (ylo) {
                const T uu1 = T(0.5) * (__ldg(U0 + c) + __ldg(U0 + c + sy));
                T uu0 = __shfl_up_sync(0xffffffffu, uu1, 1);
                if (tx == 0) uu0 = xs > 0 ? T(0.5) * (__ldg(U0 + c - 1) + __ldg(U0 + c - 1 + sy)) : T(0);
                u16.x = T(0.5) * (uu0 + uu1);
            }
            if (zlo) {
                const T uu1 = T(0.5) * (__ldg(U0 + c) + __ldg(U0 + c + sz));
                T uu0 = __shfl_up_sync(0xffffffffu, uu1, 1);
                if (tx == 0) uu0 = xs > 0 ? T(0.5) * (__ldg(U0 + c - 1) + __ldg(U0 + c - 1 + sz)) : T(0);
                u16.y = T(0.5) * (uu0 + uu1);
            }
            if (ylo || zlo) {
                const float2 f16 = vf_flux32x_x2(W2, W1, u16, c, xs, Nx, xv);
                f1 = f16.x;
                f6 = f16.y;
            }
        }
        // ---- buoyancy advection, summed as TracerMarch::step
        T db = (xs > 0) ? (T(0) + fxm) - fx : T(0) - fx;
        db = (ys > 0) ? (db + fym) - fy : db - fy;
        db = (z > 0) ? (db + fz_prev) - fz : db - fz;
        fz_prev = fz;
        // ---- vortex force, summed in the order of vortex_force_cell
        T dux = T(0), duy = T(0), duz = T(0);
        if (ylo) duy = duy - f1;
        if (xlo) dux = dux + f2;
        if (zlo) duz = duz - f3;
        if (ylo) duy = duy + f4;
        if (xlo) dux = dux - f5;
        if (zlo) duz = duz + f6;
        // ---- Bernoulli (core/bernoulli.py:14-23)
        if (xlo) dux = sub_rn(dux, sub_rn(__ldg(ke + c + 1), __ldg(ke + c)));
        if (ylo) duy = sub_rn(duy, sub_rn(__ldg(ke + c + sy), __ldg(ke + c)));
        if (zlo) {
            duz = sub_rn(duz, sub_rn(__ldg(ke + c + sz), __ldg(ke + c)));
            if (!a.euler) duz = add_rn(duz, mul_rn(a.half_dz, add_rn(__ldg(b + c + sz), __ldg(b + c))));
        }
        if (a.terms & TERM_VISC) {
            const long long cl = c;
            const int pos[3] = {z, ys, xs};
            for (int pass = 0; pass < 3; ++pass) {
                const int d = 2 - pass;
                const T cf = a.vcoef[pass];
                dux = dux + cf * lap1d(a.u[0], a.g, cl, pos[d], d);
                duy = duy + cf * lap1d(a.u[1], a.g, cl, pos[d], d);
                duz = duz + cf * lap1d(a.u[2], a.g, cl, pos[d], d);
            }
        }
        if (valid) {
            a.ds[0][c] = db;
            a.ds[1][c] = dux;
            a.ds[2][c] = duy;
            a.ds[3][c] = duz;
        }
    }
}

// advection of one passive tracer (core/tracer.py:59-72) with the same flux sharing
template <typename T, bool DIFF>
__global__ void __launch_bounds__(RZ_BX * RZ_BY) k_tracer_march(const Geom g, const T* __restrict__ Ux,
                                                                const T* __restrict__ Uy, const T* __restrict__ Uz,
                                                                const T* __restrict__ q, T* __restrict__ dq,
                                                                T kx, T ky, T kz) {
    __shared__ T sfy[RZ_BY][RZ_BX];
    const int x = blockIdx.x * RZ_BX + threadIdx.x;
    const int y = blockIdx.y * RZ_BY + threadIdx.y;
    const int z0 = blockIdx.z * RZ_ZC;
    const int z1 = min(z0 + RZ_ZC, g.N[0]) - 1;
    const bool valid = x < g.N[2] && y < g.N[1];
    const int xs = min(x, g.N[2] - 1), ys = min(y, g.N[1] - 1);
    const T* U[3] = {Uz, Uy, Ux};
    TracerMarch<T> tm;
    tm.fz_prev = z0 > 0 ? tr_flux(U[0], q, g, g.at(z0 - 1, ys, xs), z0 - 1, 0) : T(0);
    for (int z = z0; z <= z1; ++z) {
        const long long c = g.at(z, ys, xs);
        const T v = tm.step(q, U, g, c, z, ys, xs, sfy, DIFF, kx, ky, kz);
        if (valid) dq[c] = v;
    }
}

// ---------------------------------------------------------------- linear tracer schemes
// core/interpolate_tracer.f90:3-116 (coefficients: REAL(4) literals widened) and the
// linear branch of core/fortran_upwind.f90:32-61, which the reference never takes
// (`linear = .false.`, :28): selected by NylesDesc.tracer_order (param orderA).

// interpolation qp(j) (plus) or qm(j) of an odd order at 0-based position j of a line
// of n values
template <typename T, typename Q>
__device__ __forceinline__ T lin_interp_odd(int j, int n, int order, bool plus, Q q) {
    using K = LinK<T>;
    if (order == 1 || j == 0 || j == n - 1) return q(j);
    if (order == 3 || j == 1 || j == n - 2)
        return plus ? K::c1() * q(j - 1) + K::c2() * q(j) + K::c3() * q(j + 1)
                    : K::c3() * q(j - 1) + K::c2() * q(j) + K::c1() * q(j + 1);
    return plus ? K::b1() * q(j - 2) + K::b2() * q(j - 1) + K::b3() * q(j) + K::b4() * q(j + 1) + K::b5() * q(j + 2)
                : K::b5() * q(j - 2) + K::b4() * q(j - 1) + K::b3() * q(j) + K::b2() * q(j + 1) + K::b1() * q(j + 2);
}

// flux through the face to the right of 0-based cell i of a line (none at the last cell)
template <typename T, typename Q>
__device__ __forceinline__ T lin_flux(int i, int n, int order, T u, Q q) {
    using K = LinK<T>;
    if (i >= n - 1) return T(0);
    if (order == 2) return u * (T(0.5) * (q(i) + q(i + 1)));
    if (order == 4) {
        T qp;
        if (i == 0) qp = K::e2() * (q(0) + q(1)) + K::e1() * q(2);
        else if (i == n - 2) qp = K::e2() * (q(i) + q(i + 1)) + K::e1() * q(i - 1);
        else qp = K::e2() * (q(i) + q(i + 1)) + K::e1() * (q(i - 1) + q(i + 2));
        return u * qp;
    }
    const T uu = fabs(u);
    const T up = T(0.5) * (u + uu), um = T(0.5) * (u - uu);
    return up * lin_interp_odd<T>(i, n, order, true, q) + um * lin_interp_odd<T>(i + 1, n, order, false, q);
}

// -(flux divergence) of one tracer with a linear scheme, one thread per stored point,
// direction by direction in the reference's order; with `diff`, each direction's
// diffusion k*lap follows its advection (core/tracer.py:74-76)
template <typename T>
__global__ void __launch_bounds__(256) k_tracer_linear(const Geom g, const T* __restrict__ Ux,
                                                       const T* __restrict__ Uy, const T* __restrict__ Uz,
                                                       const T* __restrict__ q, T* __restrict__ dq, int order,
                                                       int diff, T kx, T ky, T kz) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= g.N[2] || y >= g.N[1] || z >= g.N[0]) return;
    const long long c = g.at(z, y, x);
    const int pos[3] = {z, y, x};
    const T* U[3] = {Uz, Uy, Ux};
    const T kc[3] = {kz, ky, kx};
    T acc = T(0);
    for (int pass = 0; pass < 3; ++pass) {
        const int d = 2 - pass;   // x, then y, then z
        const int i = pos[d], n = g.N[d];
        const long long st = g.stride(d);
        const long long base = c - (long long)i * st;
        auto Q = [&](int k) -> T { return __ldg(q + base + (long long)k * st); };
        const T fx = lin_flux<T>(i, n, order, __ldg(U[d] + c), Q);
        const T fxm = (i > 0) ? lin_flux<T>(i - 1, n, order, __ldg(U[d] + c - st), Q) : T(0);
        acc = (acc + fxm) - fx;
        if (diff) acc = acc + kc[d] * lap1d(q, g, c, i, d);
    }
    dq[c] = acc;
}

// k_rhs_les serves FP32 arrays of fewer than 2^31 cells (32-bit offsets, the largest
// one c + 3 sz + sy + 1 below 2^31); NYLES_GB300_GENERIC_RHS=1 selects k_rhs_march
// instead (the same operations; values equal to rounding). The FP64 right-hand side
// keeps k_rhs_march: it is bound by the FP64 pipe, and k_rhs_les (80 registers, 3
// blocks per SM) ran it in the same time.
template <typename T, bool BAT>
static void launch_rhs_les(dim3 grd, dim3 blk, cudaStream_t st, const RhsArgs<T>& a, const Bat& bat) {
    if constexpr (sizeof(T) == sizeof(float)) k_rhs_les<T, BAT><<<grd, blk, 0, st>>>(a, bat);
}

template <typename T>
static bool rhs32_ok(const Geom& g) {
    if (sizeof(T) != sizeof(float)) return false;
    static const bool generic = [] {
        const char* e = getenv("NYLES_GB300_GENERIC_RHS");
        return e && e[0] == '1';
    }();
    return !generic && g.vol + 4 * g.sz + g.sy + 1 < (1ll << 31);
}

bool make_geom(const NylesDesc* d, Geom* g) {
    if (!d || d->nx < 1 || d->ny < 1 || d->nz < 1 || d->nh < 0) return false;
    const int per[3] = {d->periodic_z ? 1 : 0, d->periodic_y ? 1 : 0, d->periodic_x ? 1 : 0};
    const int n[3] = {d->nz, d->ny, d->nx};
    for (int i = 0; i < 3; ++i) {
        g->n[i] = n[i];
        g->per[i] = per[i];
        g->N[i] = n[i] + (per[i] ? 2 * d->nh : 0);
        if (g->N[i] < 5) return false;   // flux1d closures need five points per line
    }
    g->nh = d->nh;
    g->sy = g->N[2];
    g->sz = (long long)g->N[1] * g->N[2];
    g->vol = g->sz * g->N[0];
    return true;
}

static dim3 grid3(const Geom& g, dim3 blk) {
    return dim3((g.N[2] + blk.x - 1) / blk.x, (g.N[1] + blk.y - 1) / blk.y, (g.N[0] + blk.z - 1) / blk.z);
}

template <typename T>
int launch_rhs(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, const ProgPtrs<T>& ds, int terms,
               cudaStream_t st, bool interior, const Bat& bat) {
    RhsArgs<T> a;
    a.g = g;
    // interior: the b and u tendencies of the periodic halo are not computed (the time
    // step refills those halos before reading them); tracers always cover every cell
    for (int k = 0; k < 3; ++k) {
        a.lo[k] = (interior && g.per[k]) ? g.nh : 0;
        a.hi[k] = (interior && g.per[k]) ? g.nh + g.n[k] : g.N[k];
    }
    a.b = s.f[NYLES_F_B];
    for (int t = 0; t < NYLES_MAX_TR; ++t) a.tr[t] = (t < d->n_tracers) ? s.f[NYLES_F_T0 + t] : nullptr;
    for (int i = 0; i < 3; ++i) {
        a.U[i] = s.f[NYLES_F_UC_I + i];
        a.W[i] = s.f[NYLES_F_VOR_I + i];
        a.u[i] = s.f[NYLES_F_U_I + i];
    }
    a.ke = s.f[NYLES_F_KE];
    for (int q = 0; q < NYLES_MAX_PROG; ++q) a.ds[q] = (q < 4 + d->n_tracers) ? ds.p[q] : nullptr;
    a.ntr = d->n_tracers;
    a.terms = terms;
    a.euler = d->model == NYLES_MODEL_EULER3D;
    a.half_dz = T(0.5 * d->dz);
    a.vcoef[0] = T(d->viscosity * d->idx2);
    a.vcoef[1] = T(d->viscosity * d->idy2);
    a.vcoef[2] = T(d->viscosity * d->idz2);
    a.kmask = d->tracer_diffusion;
    a.vf_order = d->vf_order;
    for (int q = 0; q <= NYLES_MAX_TR; ++q) {   // diff_coef[name]*ids2[direction], core/tracer.py:75
        a.kcoef[q][0] = T(d->tracer_diffusivity[q] * d->idx2);
        a.kcoef[q][1] = T(d->tracer_diffusivity[q] * d->idy2);
        a.kcoef[q][2] = T(d->tracer_diffusivity[q] * d->idz2);
    }
    if (terms & TERM_ACCUMULATE) {   // add into existing registers (vortex force alone)
        dim3 blk(32, 2, 2);
        k_rhs<T><<<grid3(g, blk), blk, 0, st>>>(a);
        note_launch();
        return cuda_status(cudaGetLastError(), "rhs kernel");
    }
    const dim3 blk(RZ_BX, RZ_BY, 1);
    const dim3 grd((g.N[2] + RZ_BX - 1) / RZ_BX, (g.N[1] + RZ_BY - 1) / RZ_BY, (g.N[0] + RZ_ZC - 1) / RZ_ZC);
    const dim3 grd_box((a.hi[2] - a.lo[2] + RZ_BX - 1) / RZ_BX, (a.hi[1] - a.lo[1] + RZ_BY - 1) / RZ_BY,
                       (a.hi[0] - a.lo[0] + RZ_ZC - 1) / RZ_ZC);
    const int order = d->tracer_order;
    const dim3 lblk(32, 4, 2);
    auto tracer_linear = [&](const T* q, T* dq, int qi) {
        const bool diff = (terms & TERM_TRDIFF) && ((d->tracer_diffusion >> qi) & 1);
        const T* kc = a.kcoef[qi];
        k_tracer_linear<T><<<grid3(g, lblk), lblk, 0, st>>>(g, a.U[0], a.U[1], a.U[2], q, dq, order, diff ? 1 : 0,
                                                            kc[0], kc[1], kc[2]);
        note_launch();
    };
    if (d->model == NYLES_MODEL_ADVECTION) {
        // Advection.rhs (core/model_advection.py:59-61): b only; the velocity registers
        // are not touched (the reference never writes them)
        if (order > 0) {
            tracer_linear(a.b, a.ds[0], 0);
        } else {
            const T* kc = a.kcoef[0];
            if ((terms & TERM_TRDIFF) && (d->tracer_diffusion & 1))
                k_tracer_march<T, true><<<grd, blk, 0, st>>>(g, a.U[0], a.U[1], a.U[2], a.b, a.ds[0], kc[0], kc[1],
                                                             kc[2]);
            else
                k_tracer_march<T, false><<<grd, blk, 0, st>>>(g, a.U[0], a.U[1], a.U[2], a.b, a.ds[0], T(0), T(0),
                                                              T(0));
            note_launch();
        }
        return cuda_status(cudaGetLastError(), "rhs kernel");
    }
    const bool linear_tr = (terms & TERM_TRACER) && order > 0;
    if (linear_tr) terms &= ~TERM_TRACER;   // b's tendency comes from k_tracer_linear after the march
    const bool tr = (terms & TERM_TRACER) != 0, vf = (terms & TERM_VF) != 0;
    const bool bdiff = tr && (terms & TERM_TRDIFF) && (d->tracer_diffusion & 1);
    const bool lin = vf && d->vf_order > 0;
    if (bat.tab) {   // batched: buoyancy advection, WENO vortex force, no buoyancy diffusion
        if (!(tr && vf && !bdiff && !lin && !linear_tr && d->n_tracers == 0 && d->model != NYLES_MODEL_ADVECTION)) {
            set_error("batched right-hand side: only buoyancy advection with the WENO vortex force and no tracers");
            return NYLES_UNSUPPORTED;
        }
        const dim3 gb(grd_box.x, grd_box.y, grd_box.z * bat.nrun);
        if (rhs32_ok<T>(g)) launch_rhs_les<T, true>(gb, blk, st, a, bat);
        else k_rhs_march<T, true, 1, false, true><<<gb, blk, 0, st>>>(a, bat);
        note_launch();
        return cuda_status(cudaGetLastError(), "rhs kernel");
    }
    if (lin) {   // the linear vortex force (opt-in)
        if (tr && bdiff) k_rhs_march<T, true, 2, true><<<grd_box, blk, 0, st>>>(a);
        else if (tr) k_rhs_march<T, true, 2, false><<<grd_box, blk, 0, st>>>(a);
        else k_rhs_march<T, false, 2, false><<<grd_box, blk, 0, st>>>(a);
    } else if (tr && vf && bdiff) k_rhs_march<T, true, 1, true><<<grd_box, blk, 0, st>>>(a);
    else if (tr && vf && rhs32_ok<T>(g)) launch_rhs_les<T, false>(grd_box, blk, st, a, Bat());
    else if (tr && vf) k_rhs_march<T, true, 1, false><<<grd_box, blk, 0, st>>>(a);
    else if (tr && bdiff) k_rhs_march<T, true, 0, true><<<grd_box, blk, 0, st>>>(a);
    else if (tr) k_rhs_march<T, true, 0, false><<<grd_box, blk, 0, st>>>(a);
    else if (vf) k_rhs_march<T, false, 1, false><<<grd_box, blk, 0, st>>>(a);
    else k_rhs_march<T, false, 0, false><<<grd_box, blk, 0, st>>>(a);
    note_launch();
    if (linear_tr) {
        tracer_linear(a.b, a.ds[0], 0);
        for (int t = 0; t < d->n_tracers; ++t) tracer_linear(a.tr[t], a.ds[4 + t], t + 1);
        return cuda_status(cudaGetLastError(), "rhs kernel");
    }
    for (int t = 0; t < d->n_tracers; ++t) {
        if (tr) {
            const T* kc = a.kcoef[t + 1];
            if ((terms & TERM_TRDIFF) && ((d->tracer_diffusion >> (t + 1)) & 1))
                k_tracer_march<T, true><<<grd, blk, 0, st>>>(g, a.U[0], a.U[1], a.U[2], a.tr[t], a.ds[4 + t],
                                                             kc[0], kc[1], kc[2]);
            else
                k_tracer_march<T, false><<<grd, blk, 0, st>>>(g, a.U[0], a.U[1], a.U[2], a.tr[t], a.ds[4 + t],
                                                              T(0), T(0), T(0));
            note_launch();
        } else {   // Euler3d: tracers are not advected, their tendency is zero (reset_state)
            cudaMemsetAsync(a.ds[4 + t], 0, sizeof(T) * g.vol, st);
        }
    }
    return cuda_status(cudaGetLastError(), "rhs kernel");
}

// ---------------------------------------------------------------- time-scheme updates
template <typename T>
struct UpdArgs {
    long long vol;
    int nprog;
    int kind;
    T k1, k2;         // the stage's coefficients, rounded to T on the host (see launch_update)
    T* s[NYLES_MAX_PROG];
    T* a[NYLES_MAX_PROG];
    T* b[NYLES_MAX_PROG];
    T* c[NYLES_MAX_PROG];
};

// numpy's evaluation order of core/timescheme.py:113-221, one rounding per operation;
// one prognostic field after the other, a grid-stride loop over its cells
template <typename T, int KIND>
__device__ __forceinline__ void update_field(T* __restrict__ s, const T* __restrict__ a, T* __restrict__ b,
                                             T* __restrict__ c, long long vol, T k1, T k2) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < vol; i += stride) {
        if (KIND == UPD_EULER) {   // s += dt*ds
            s[i] = add_rn(s[i], mul_rn(k1, a[i]));
        } else if (KIND == UPD_RK3_2) {   // s += (dt/4.)*(ds1-3*ds0)
            const T t2 = sub_rn(b[i], mul_rn(T(3), a[i]));
            s[i] = add_rn(s[i], mul_rn(k1, t2));
        } else if (KIND == UPD_RK3_3) {   // s += (dt/12.)*(8*ds2-ds0-ds1)
            const T t3 = sub_rn(sub_rn(mul_rn(T(8), c[i]), a[i]), b[i]);
            s[i] = add_rn(s[i], mul_rn(k1, t3));
        } else if (KIND == UPD_LF_FIRST) {   // sn = s; sb = s; s += dt*ds  (a = ds, b = sb, c = sn)
            const T v = s[i];
            c[i] = v;
            b[i] = v;
            s[i] = add_rn(v, mul_rn(k1, a[i]));
        } else if (KIND == UPD_LF_PRED) {   // sn = s; s = sb + 2dt*ds; s = (1/12)*(5s + 8sn - sb); sb = sn
            const T sn = s[i];
            const T sb = b[i];
            const T lf = add_rn(sb, mul_rn(k1, a[i]));
            const T t4 = sub_rn(add_rn(mul_rn(T(5), lf), mul_rn(T(8), sn)), sb);
            s[i] = mul_rn(k2, t4);
            c[i] = sn;
            b[i] = sn;
        } else {   // UPD_LF_CORR: s = sn + dt*ds
            s[i] = add_rn(c[i], mul_rn(k1, a[i]));
        }
    }
}

template <typename T, int KIND>
__global__ void k_update(const UpdArgs<T> p, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    for (int q = 0; q < p.nprog; ++q)
        update_field<T, KIND>(bshift(p.s[q], dlt), bshift(p.a[q], dlt), bshift(p.b[q], dlt), bshift(p.c[q], dlt),
                              p.vol, p.k1, p.k2);
}

template <typename T>
int launch_update(const Geom& g, int nprog, const ProgPtrs<T>& s, const ProgPtrs<T>& a, const ProgPtrs<T>& b,
                  const ProgPtrs<T>& c, int kind, double dt, cudaStream_t st, const Bat& bat) {
    UpdArgs<T> p;
    p.vol = g.vol;
    p.nprog = nprog;
    p.kind = kind;
    // the coefficients numpy forms in double (dt/4., dt/12., 2*dt, 1/12.), rounded to T
    // once here instead of per cell on the device's FP64 pipe
    p.k1 = T(dt);
    p.k2 = T(0);
    if (kind == UPD_RK3_2) p.k1 = T(dt / 4.0);
    else if (kind == UPD_RK3_3) p.k1 = T(dt / 12.0);
    else if (kind == UPD_LF_PRED) { p.k1 = T(2.0 * dt); p.k2 = T(1.0 / 12.0); }
    for (int q = 0; q < NYLES_MAX_PROG; ++q) {
        p.s[q] = s.p[q]; p.a[q] = a.p[q]; p.b[q] = b.p[q]; p.c[q] = c.p[q];
    }
    long long blocks = (g.vol + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    const dim3 grd((unsigned)blocks, 1, bat.tab ? bat.nrun : 1);
    switch (kind) {
        case UPD_EULER: k_update<T, UPD_EULER><<<grd, 256, 0, st>>>(p, bat); break;
        case UPD_RK3_2: k_update<T, UPD_RK3_2><<<grd, 256, 0, st>>>(p, bat); break;
        case UPD_RK3_3: k_update<T, UPD_RK3_3><<<grd, 256, 0, st>>>(p, bat); break;
        case UPD_LF_FIRST: k_update<T, UPD_LF_FIRST><<<grd, 256, 0, st>>>(p, bat); break;
        case UPD_LF_PRED: k_update<T, UPD_LF_PRED><<<grd, 256, 0, st>>>(p, bat); break;
        case UPD_LF_CORR: k_update<T, UPD_LF_CORR><<<grd, 256, 0, st>>>(p, bat); break;
        default: set_error("unknown update kind"); return NYLES_BAD_ARG;
    }
    note_launch();
    return cuda_status(cudaGetLastError(), "update kernel");
}

// ---------------------------------------------------------------- periodic halo fill
// core/mpi/halo.py:140-178 for one rank: each halo cell receives its periodic image.
// The halo is enumerated as six disjoint slabs (z-low/high over everything, then
// y-low/high over interior z, then x-low/high over interior z and y).
struct FillSlabs {
    int lo[6][3], ext[6][3];
    long long count[6];
    int nslab;
};

template <typename T>
struct FillArgs {
    Geom g;
    FillSlabs sl;
    T* f[8];
    int nf;
};

template <typename T>
__global__ void k_fill(const FillArgs<T> a, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    const int s = blockIdx.y;
    if (s >= a.sl.nslab) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.sl.count[s]) return;
    const int ex = a.sl.ext[s][2], ey = a.sl.ext[s][1];
    const int x = a.sl.lo[s][2] + (int)(i % ex);
    const int y = a.sl.lo[s][1] + (int)((i / ex) % ey);
    const int z = a.sl.lo[s][0] + (int)(i / ((long long)ex * ey));
    const Geom& g = a.g;
    const long long dst = g.at(z, y, x);
    const long long src = g.at(g.wrap(0, z), g.wrap(1, y), g.wrap(2, x));
    for (int k = 0; k < a.nf; ++k) {
        T* f = bshift(a.f[k], dlt);
        f[dst] = f[src];
    }
}

static FillSlabs make_slabs(const Geom& g) {
    FillSlabs s{};
    int n = 0;
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { lo[d] = g.per[d] ? g.nh : 0; hi[d] = g.per[d] ? g.nh + g.n[d] : g.N[d]; }
    for (int d = 0; d < 3; ++d) {
        if (!g.per[d]) continue;
        for (int side = 0; side < 2; ++side) {
            int l[3], e[3];
            for (int k = 0; k < 3; ++k) {
                if (k < d) { l[k] = lo[k]; e[k] = hi[k] - lo[k]; }
                else if (k > d) { l[k] = 0; e[k] = g.N[k]; }
                else { l[k] = side ? hi[k] : 0; e[k] = g.nh; }
            }
            for (int k = 0; k < 3; ++k) { s.lo[n][k] = l[k]; s.ext[n][k] = e[k]; }
            s.count[n] = (long long)e[0] * e[1] * e[2];
            ++n;
        }
    }
    s.nslab = n;
    return s;
}

template <typename T>
int launch_fill(const Geom& g, T* const* fields, int nf, cudaStream_t st, const Bat& bat) {
    FillArgs<T> a;
    a.g = g;
    a.sl = make_slabs(g);
    if (a.sl.nslab == 0) return NYLES_OK;
    long long mx = 0;
    for (int s = 0; s < a.sl.nslab; ++s) mx = a.sl.count[s] > mx ? a.sl.count[s] : mx;
    for (int base = 0; base < nf; base += 8) {
        a.nf = (nf - base) < 8 ? (nf - base) : 8;
        for (int k = 0; k < a.nf; ++k) a.f[k] = fields[base + k];
        dim3 grd((unsigned)((mx + 255) / 256), a.sl.nslab, bat.tab ? bat.nrun : 1);
        k_fill<T><<<grd, 256, 0, st>>>(a, bat);
        note_launch();
    }
    return cuda_status(cudaGetLastError(), "fill kernel");
}

// ---------------------------------------------------------------- divergence
// core/projection.py:16-29 (fortran_bernoulli.f90:61-97) on U = u*ids2
// (core/cov_to_contra.py:16-18), evaluated at the periodic image of each cell because
// core/mgfordriver.py:70 fills the halo of div before the solve.
// The divergence and the projection correction run one thread per (y, x) column of the
// array and PJ_ZC cells in z: the column's wrapped position and interior offset are
// computed once.
constexpr int PJ_BX = 32, PJ_BY = 8, PJ_ZC = 8;
static inline dim3 grid_pj(const Geom& g) {
    return dim3((unsigned)((g.N[2] + PJ_BX - 1) / PJ_BX), (unsigned)((g.N[1] + PJ_BY - 1) / PJ_BY),
                (unsigned)((g.N[0] + PJ_ZC - 1) / PJ_ZC));
}

template <typename T, typename TB>
__global__ void __launch_bounds__(PJ_BX * PJ_BY) k_div(const Geom g, const T* __restrict__ ux, const T* __restrict__ uy,
                                                       const T* __restrict__ uz, TB idx2, TB idy2, TB idz2,
                                                       T* __restrict__ div, TB* __restrict__ mgb) {
    const int x = blockIdx.x * PJ_BX + threadIdx.x;
    const int y = blockIdx.y * PJ_BY + threadIdx.y;
    if (x >= g.N[2] || y >= g.N[1]) return;
    const int z0 = blockIdx.z * PJ_ZC, z1 = min(z0 + PJ_ZC, g.N[0]);
    const int yy = g.wrap(1, y), xx = g.wrap(2, x);
    const bool own_xy = yy == y && xx == x;
    const long long cxy = (long long)yy * g.sy + xx;
    const long long ixy = (long long)(yy - (g.per[1] ? g.nh : 0)) * g.n[2] + (xx - (g.per[2] ? g.nh : 0));
    for (int z = z0; z < z1; ++z) {
        const int zz = g.wrap(0, z);
        const long long c = (long long)zz * g.sz + cxy;
        TB acc;
        {
            TB U0 = mul_rn(TB(ux[c]), idx2);
            acc = (xx == 0) ? U0 : sub_rn(U0, mul_rn(TB(ux[c - 1]), idx2));
        }
        {
            TB V0 = mul_rn(TB(uy[c]), idy2);
            acc = (yy == 0) ? add_rn(acc, V0) : add_rn(acc, sub_rn(V0, mul_rn(TB(uy[c - g.sy]), idy2)));
        }
        {
            TB W0 = mul_rn(TB(uz[c]), idz2);
            acc = (zz == 0) ? add_rn(acc, W0) : add_rn(acc, sub_rn(W0, mul_rn(TB(uz[c - g.sz]), idz2)));
        }
        div[g.at(z, y, x)] = T(acc);
        if (own_xy && zz == z) {
            const int iz = zz - (g.per[0] ? g.nh : 0);
            mgb[(long long)iz * g.n[1] * g.n[2] + ixy] = acc;
        }
    }
}

// mixed precision: the same divergence of the FP32 velocity carried as a float pair
// (products by the metric factor and differences are exact to ~2^-48), written to the
// multigrid right-hand side as (hi, lo); the model's div field gets hi + lo rounded.
// One column per thread, as k_div.

// (a - b) * (s.hi + s.lo) as a float pair: the difference of two floats is exact as a
// pair (TwoSum), then one pair product (both within ~2^-48 of the exact value)
__device__ __forceinline__ float2 ddiff_mul(float a, float b, float2 s) {
    float d, e;
    two_sum(a, -b, d, e);
    return df_mul(make_float2(d, e), s);
}

__global__ void __launch_bounds__(PJ_BX * PJ_BY) k_div_df(const Geom g, const float* __restrict__ ux,
                                                          const float* __restrict__ uy, const float* __restrict__ uz,
                                                          float2 idx2, float2 idy2, float2 idz2,
                                                          float* __restrict__ div, float2* __restrict__ mgb,
                                                          const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    ux = bshift(ux, dlt);
    uy = bshift(uy, dlt);
    uz = bshift(uz, dlt);
    div = bshift(div, dlt);
    mgb = bshift(mgb, dlt);
    const int x = blockIdx.x * PJ_BX + threadIdx.x;
    const int y = blockIdx.y * PJ_BY + threadIdx.y;
    if (x >= g.N[2] || y >= g.N[1]) return;
    const int z0 = bz * PJ_ZC, z1 = min(z0 + PJ_ZC, g.N[0]);
    const int yy = g.wrap(1, y), xx = g.wrap(2, x);
    const bool own_xy = yy == y && xx == x;
    const long long cxy = (long long)yy * g.sy + xx;
    const long long ixy = (long long)(yy - (g.per[1] ? g.nh : 0)) * g.n[2] + (xx - (g.per[2] ? g.nh : 0));
    for (int z = z0; z < z1; ++z) {
        const int zz = g.wrap(0, z);
        const long long c = (long long)zz * g.sz + cxy;
        float2 acc = ddiff_mul(ux[c], xx != 0 ? ux[c - 1] : 0.f, idx2);
        acc = df_add(acc, ddiff_mul(uy[c], yy != 0 ? uy[c - g.sy] : 0.f, idy2));
        acc = df_add(acc, ddiff_mul(uz[c], zz != 0 ? uz[c - g.sz] : 0.f, idz2));
        div[g.at(z, y, x)] = df_value(acc);
        if (own_xy && zz == z) {
            const int iz = zz - (g.per[0] ? g.nh : 0);
            mgb[(long long)iz * g.n[1] * g.n[2] + ixy] = acc;
        }
    }
}

template <typename T, typename TB>
int launch_div(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, TB* mg_b, cudaStream_t st) {
    k_div<T, TB><<<grid_pj(g), dim3(PJ_BX, PJ_BY), 0, st>>>(g, s.f[NYLES_F_U_I], s.f[NYLES_F_U_J], s.f[NYLES_F_U_K],
                                                 TB(d->idx2), TB(d->idy2), TB(d->idz2), s.f[NYLES_F_DIV], mg_b);
    note_launch();
    return cuda_status(cudaGetLastError(), "div kernel");
}

int launch_div_df(const NylesDesc* d, const Geom& g, const StencilPtrs<float>& s, float2* mg_b, cudaStream_t st,
                  const Bat& bat) {
    dim3 grd = grid_pj(g);
    if (bat.tab) grd.z *= bat.nrun;
    k_div_df<<<grd, dim3(PJ_BX, PJ_BY), 0, st>>>(g, s.f[NYLES_F_U_I], s.f[NYLES_F_U_J], s.f[NYLES_F_U_K],
                                                 df_split(d->idx2), df_split(d->idy2), df_split(d->idz2),
                                                 s.f[NYLES_F_DIV], mg_b, bat);
    note_launch();
    return cuda_status(cudaGetLastError(), "div kernel");
}

// ---------------------------------------------------------------- projection correction
// p = x*dx**2 (core/mgfordriver.py:78) on every cell (halo = periodic image) and
// u_i -= p(i+1)-p(i) (core/projection.py:84-87 via fortran_bernoulli.f90:2-26) on the
// interior cells. The correction reads no velocity neighbour, so it runs in place;
// the halo of u is filled afterwards as core/model_les.py:110 does.
template <typename T, typename TP>
struct CorrArgs {
    Geom g;
    T* u[3];
    const TP* x;      // pressure solution, interior cells (nz, ny, nx)
    T* p;
    double dx2;
};

template <typename T, typename TP>
__global__ void __launch_bounds__(PJ_BX * PJ_BY) k_correct(const CorrArgs<T, TP> a) {
    const Geom& g = a.g;
    const int x = blockIdx.x * PJ_BX + threadIdx.x;
    const int y = blockIdx.y * PJ_BY + threadIdx.y;
    if (x >= g.N[2] || y >= g.N[1]) return;
    const int z0 = blockIdx.z * PJ_ZC, z1 = min(z0 + PJ_ZC, g.N[0]);
    const int oz = g.per[0] ? g.nh : 0, oy = g.per[1] ? g.nh : 0, ox = g.per[2] ? g.nh : 0;
    const int yy = g.wrap(1, y), xx = g.wrap(2, x);
    const bool own_xy = yy == y && xx == x;
    const long long n2 = g.n[2], sxy = (long long)g.n[1] * n2;
    // interior index of the column's image and of its x + 1 and y + 1 neighbours' images
    const long long ixy = (long long)(yy - oy) * n2 + (xx - ox);
    const bool hx = x < g.N[2] - 1, hy = y < g.N[1] - 1;
    const long long ixy_x = hx ? (long long)(yy - oy) * n2 + (g.wrap(2, x + 1) - ox) : ixy;
    const long long ixy_y = hy ? (long long)(g.wrap(1, y + 1) - oy) * n2 + (xx - ox) : ixy;
    const TP dx2 = TP(a.dx2);
    for (int z = z0; z < z1; ++z) {
        const long long c = g.at(z, y, x);
        const int zz = g.wrap(0, z);
        const long long iz = (long long)(zz - oz) * sxy;
        const TP p0 = mul_rn(a.x[iz + ixy], dx2);
        a.p[c] = T(p0);
        if (!own_xy || zz != z) continue;   // halo: filled later
        if (hx) a.u[0][c] = T(sub_rn(TP(a.u[0][c]), sub_rn(mul_rn(a.x[iz + ixy_x], dx2), p0)));
        if (hy) a.u[1][c] = T(sub_rn(TP(a.u[1][c]), sub_rn(mul_rn(a.x[iz + ixy_y], dx2), p0)));
        if (z < g.N[0] - 1) {
            const long long iz1 = (long long)(g.wrap(0, z + 1) - oz) * sxy;
            a.u[2][c] = T(sub_rn(TP(a.u[2][c]), sub_rn(mul_rn(a.x[iz1 + ixy], dx2), p0)));
        }
    }
}

template <typename T, typename TP>
int launch_correct(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, const TP* mg_x, double dx2,
                   cudaStream_t st) {
    (void)d;
    CorrArgs<T, TP> a;
    a.g = g;
    for (int i = 0; i < 3; ++i) a.u[i] = s.f[NYLES_F_U_I + i];
    a.x = mg_x;
    a.p = s.f[NYLES_F_P];
    a.dx2 = dx2;
    k_correct<T, TP><<<grid_pj(g), dim3(PJ_BX, PJ_BY), 0, st>>>(a);
    note_launch();
    return cuda_status(cudaGetLastError(), "correct kernel");
}

// mixed precision: the same correction from the float-pair solution; differences of
// neighbouring pressures and the dx^2 scaling are taken on the pairs, then rounded.
struct CorrDfArgs {
    Geom g;
    float* u[3];
    const float2* x;
    float* p;
    float2 dx2;
};

// one thread per (y, x) column of the array, PJ_ZC cells in z (as k_div_df)
__global__ void __launch_bounds__(PJ_BX * PJ_BY) k_correct_df(const CorrDfArgs a0, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    CorrDfArgs a = a0;
    if (dlt) {
        for (int i = 0; i < 3; ++i) a.u[i] = bshift(a.u[i], dlt);
        a.x = bshift(a.x, dlt);
        a.p = bshift(a.p, dlt);
    }
    const Geom& g = a.g;
    const int x = blockIdx.x * PJ_BX + threadIdx.x;
    const int y = blockIdx.y * PJ_BY + threadIdx.y;
    if (x >= g.N[2] || y >= g.N[1]) return;
    // distinct arrays: the loads of the next cell need not wait for this cell's stores
    const float2* __restrict__ X = a.x;
    float* __restrict__ P = a.p;
    float* __restrict__ U0 = a.u[0];
    float* __restrict__ U1 = a.u[1];
    float* __restrict__ U2 = a.u[2];
    const int z0 = bz * PJ_ZC, z1 = min(z0 + PJ_ZC, g.N[0]);
    const int oz = g.per[0] ? g.nh : 0, oy = g.per[1] ? g.nh : 0, ox = g.per[2] ? g.nh : 0;
    const int yy = g.wrap(1, y), xx = g.wrap(2, x);
    const bool own_xy = yy == y && xx == x;
    const long long n2 = g.n[2], sxy = (long long)g.n[1] * n2;
    // interior index of the column's image and of its x + 1 and y + 1 neighbours' images
    const long long ixy = (long long)(yy - oy) * n2 + (xx - ox);
    const bool hx = x < g.N[2] - 1, hy = y < g.N[1] - 1;
    const long long ixy_x = hx ? (long long)(yy - oy) * n2 + (g.wrap(2, x + 1) - ox) : ixy;
    const long long ixy_y = hy ? (long long)(g.wrap(1, y + 1) - oy) * n2 + (xx - ox) : ixy;
    for (int z = z0; z < z1; ++z) {
        const long long c = g.at(z, y, x);
        const int zz = g.wrap(0, z);
        const long long iz = (long long)(zz - oz) * sxy;
        const float2 p0 = X[iz + ixy];
        P[c] = df_value(df_mul(p0, a.dx2));
        if (!own_xy || zz != z) continue;   // halo: filled later
        const float2 np0 = df_neg(p0);
        if (hx) U0[c] = __fsub_rn(U0[c], df_value(df_mul(df_add(X[iz + ixy_x], np0), a.dx2)));
        if (hy) U1[c] = __fsub_rn(U1[c], df_value(df_mul(df_add(X[iz + ixy_y], np0), a.dx2)));
        if (z < g.N[0] - 1) {
            const long long iz1 = (long long)(g.wrap(0, z + 1) - oz) * sxy;
            U2[c] = __fsub_rn(U2[c], df_value(df_mul(df_add(X[iz1 + ixy], np0), a.dx2)));
        }
    }
}

int launch_correct_df(const Geom& g, const StencilPtrs<float>& s, const float2* mg_x, double dx2, cudaStream_t st,
                      const Bat& bat) {
    CorrDfArgs a;
    a.g = g;
    for (int i = 0; i < 3; ++i) a.u[i] = s.f[NYLES_F_U_I + i];
    a.x = mg_x;
    a.p = s.f[NYLES_F_P];
    a.dx2 = df_split(dx2);
    dim3 grd = grid_pj(g);
    if (bat.tab) grd.z *= bat.nrun;
    k_correct_df<<<grd, dim3(PJ_BX, PJ_BY), 0, st>>>(a, bat);
    note_launch();
    return cuda_status(cudaGetLastError(), "correct kernel");
}

// ---------------------------------------------------------------- diagnostics
// From the corrected, halo-filled u: U = u*ids2 (core/cov_to_contra.py:4-20),
// vorticity (core/vorticity.py:26-34 -> fortran_vorticity.f90:16-26 in each
// orientation, Coriolis added to vor_k), kinetic energy (core/kinenergy.py:17-24 ->
// fortran_kinenergy.f90:47-53). Each cell evaluates at its periodic image, which is
// what the fills of vor and ke (core/model_les.py:126-127) leave in the halo.
template <typename T>
struct DiagArgs {
    Geom g;
    const T* u[3];
    T* U[3];
    T* W[3];
    T* ke;
    T ids2[3];
    T kec[3];         // (0.5*ids2)*0.5
    T fparam;
    int nonlinear;
};

template <typename T>
__global__ void __launch_bounds__(256) k_diag(const DiagArgs<T> a0, const Bat bat = Bat()) {
    int bz;
    long long dlt;
    if (!batch_enter(bat, bz, dlt)) return;
    DiagArgs<T> a = a0;
    if (dlt) {
        for (int i = 0; i < 3; ++i) {
            a.u[i] = bshift(a.u[i], dlt);
            a.U[i] = bshift(a.U[i], dlt);
            a.W[i] = bshift(a.W[i], dlt);
        }
        a.ke = bshift(a.ke, dlt);
    }
    const Geom& g = a.g;
    const int x0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int y0 = blockIdx.y * blockDim.y + threadIdx.y;
    const int z0 = bz * blockDim.z + threadIdx.z;
    if (x0 >= g.N[2] || y0 >= g.N[1] || z0 >= g.N[0]) return;
    const long long c0 = g.at(z0, y0, x0);
    const T* __restrict__ ux = a.u[0];
    const T* __restrict__ uy = a.u[1];
    const T* __restrict__ uz = a.u[2];
    const T ui = ux[c0], uj = uy[c0], uk = uz[c0];   // u is filled: value at c0 == value at the image
    a.U[0][c0] = mul_rn(ui, a.ids2[0]);
    a.U[1][c0] = mul_rn(uj, a.ids2[1]);
    a.U[2][c0] = mul_rn(uk, a.ids2[2]);
    if (!a.nonlinear) return;
    const int z = g.wrap(0, z0), y = g.wrap(1, y0), x = g.wrap(2, x0);
    const long long c = g.at(z, y, x);
    const int Nz = g.N[0], Ny = g.N[1], Nx = g.N[2];
    T wi = T(0), wj = T(0), wk = T(0);
    if (z < Nz - 1 && y < Ny - 1) wi = add_rn(sub_rn(sub_rn(uz[c + g.sy], uk), uy[c + g.sz]), uj);
    if (x < Nx - 1 && z < Nz - 1) wj = add_rn(sub_rn(sub_rn(ux[c + g.sz], ui), uz[c + 1]), uk);
    if (y < Ny - 1 && x < Nx - 1) {
        wk = add_rn(sub_rn(sub_rn(uy[c + 1], uj), ux[c + g.sy]), ui);
        if (a.fparam > T(0)) wk = add_rn(wk, a.fparam);
    }
    a.W[0][c0] = wi; a.W[1][c0] = wj; a.W[2][c0] = wk;
    T ke = T(0);
    if (x >= 1) { const T m = ux[c - 1]; ke = add_rn(ke, mul_rn(a.kec[0], add_rn(mul_rn(ui, ui), mul_rn(m, m)))); }
    if (y >= 1) { const T m = uy[c - g.sy]; ke = add_rn(ke, mul_rn(a.kec[1], add_rn(mul_rn(uj, uj), mul_rn(m, m)))); }
    if (z >= 1) { const T m = uz[c - g.sz]; ke = add_rn(ke, mul_rn(a.kec[2], add_rn(mul_rn(uk, uk), mul_rn(m, m)))); }
    a.ke[c0] = ke;
}

template <typename T>
int launch_diag(const NylesDesc* d, const Geom& g, const StencilPtrs<T>& s, int nonlinear, cudaStream_t st,
                const Bat& bat) {
    DiagArgs<T> a;
    a.g = g;
    for (int i = 0; i < 3; ++i) {
        a.u[i] = s.f[NYLES_F_U_I + i];
        a.U[i] = s.f[NYLES_F_UC_I + i];
        a.W[i] = s.f[NYLES_F_VOR_I + i];
    }
    a.ke = s.f[NYLES_F_KE];
    const double ids2[3] = {d->idx2, d->idy2, d->idz2};
    for (int i = 0; i < 3; ++i) {
        a.ids2[i] = T(ids2[i]);
        a.kec[i] = T((0.5 * ids2[i]) * 0.5);
    }
    a.fparam = T(d->fparam);
    a.nonlinear = nonlinear;
    dim3 blk(32, 4, 2);
    dim3 grd = grid3(g, blk);
    if (bat.tab) grd.z *= bat.nrun;
    k_diag<T><<<grd, blk, 0, st>>>(a, bat);
    note_launch();
    return cuda_status(cudaGetLastError(), "diag kernel");
}

// ---------------------------------------------------------------- CFL reduction
// max over all stored points of U^2+V^2+W^2, core/nyles.py:241-251 (max is exact
// whatever the reduction order)
template <typename T>
__global__ void __launch_bounds__(256) k_max_U2(const long long vol, const T* __restrict__ U,
                                                const T* __restrict__ V, const T* __restrict__ W,
                                                double* __restrict__ partial) {
    double m = 0.0;
    bool any_nan = false;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < vol; i += stride) {
        const double a = U[i], b = V[i], c = W[i];
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
        if (s != s) any_nan = true;
        m = fmax(m, s);
    }
    __shared__ double sm[8];
    __shared__ int snan;
    if (threadIdx.x == 0) snan = 0;
    __syncthreads();
    if (any_nan) snan = 1;
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        v = warp_max(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = snan ? __longlong_as_double(0x7ff8000000000000ULL) : v;
    }
}

__global__ void k_max_final(const double* __restrict__ partial, int n, double* out) {
    double m = 0.0;
    bool nan = false;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double v = partial[i];
        if (v != v) nan = true;
        m = fmax(m, v);
    }
    __shared__ double sm[32];
    __shared__ int snan;
    if (threadIdx.x == 0) snan = 0;
    __syncthreads();
    if (nan) snan = 1;
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        v = warp_max(v);
        if (threadIdx.x == 0) out[0] = snan ? __longlong_as_double(0x7ff8000000000000ULL) : v;
    }
}

template <typename T>
int launch_max_U2(const Geom& g, const StencilPtrs<T>& s, double* partial, int npartial, double* out,
                  cudaStream_t st) {
    k_max_U2<T><<<npartial, 256, 0, st>>>(g.vol, s.f[NYLES_F_UC_I], s.f[NYLES_F_UC_J], s.f[NYLES_F_UC_K], partial);
    k_max_final<<<1, 1024, 0, st>>>(partial, npartial, out);
    note_launch(2);
    return cuda_status(cudaGetLastError(), "max_U2 kernel");
}

// ---------------------------------------------------------------- vortex-force work
// core/online_diag.py:27-35: work(p) = sum over d = i, j, k (in that order) of
// (U_d F_d / 2)(p) + (U_d F_d / 2)(p - e_d) where the index along d is >= 1; the products
// and the sum of work over the box are taken in FP64 whatever the storage type. Each
// block of a fixed grid strides over the array in a fixed order, so the partial sums,
// and the total, are the same on every run.
template <typename T>
__global__ void __launch_bounds__(256) k_vfwork(Geom g, const T* __restrict__ U, const T* __restrict__ V,
                                                const T* __restrict__ W, const T* __restrict__ FU,
                                                const T* __restrict__ FV, const T* __restrict__ FW,
                                                T* __restrict__ work, VfBox box, double* __restrict__ partial) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int Nx = g.N[2], Ny = g.N[1];
    double acc = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < g.vol; q += stride) {
        const int i = (int)(q % Nx);
        const long long r = q / Nx;
        const int j = (int)(r % Ny);
        const int k = (int)(r / Ny);
        double w = 0.0;
        if (i >= 1) {
            const double a = __dmul_rn(__dmul_rn((double)U[q], (double)FU[q]), 0.5);
            const double b = __dmul_rn(__dmul_rn((double)U[q - 1], (double)FU[q - 1]), 0.5);
            w = __dadd_rn(w, __dadd_rn(a, b));
        }
        if (j >= 1) {
            const double a = __dmul_rn(__dmul_rn((double)V[q], (double)FV[q]), 0.5);
            const double b = __dmul_rn(__dmul_rn((double)V[q - g.sy], (double)FV[q - g.sy]), 0.5);
            w = __dadd_rn(w, __dadd_rn(a, b));
        }
        if (k >= 1) {
            const double a = __dmul_rn(__dmul_rn((double)W[q], (double)FW[q]), 0.5);
            const double b = __dmul_rn(__dmul_rn((double)W[q - g.sz], (double)FW[q - g.sz]), 0.5);
            w = __dadd_rn(w, __dadd_rn(a, b));
        }
        work[q] = (T)w;
        if (k >= box.lo[0] && k < box.hi[0] && j >= box.lo[1] && j < box.hi[1] && i >= box.lo[2] && i < box.hi[2])
            acc += w;
    }
    __shared__ double sm[8];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void k_sum_final(const double* __restrict__ partial, int n, double* out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    __shared__ double sm[32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) out[0] = v;
    }
}

template <typename T>
int launch_vfwork(const Geom& g, const StencilPtrs<T>& s, const ProgPtrs<T>& ds, const VfBox& box, double* partial,
                  int npartial, double* out, cudaStream_t st) {
    k_vfwork<T><<<npartial, 256, 0, st>>>(g, s.f[NYLES_F_UC_I], s.f[NYLES_F_UC_J], s.f[NYLES_F_UC_K], ds.p[1],
                                          ds.p[2], ds.p[3], s.f[NYLES_F_WORK], box, partial);
    k_sum_final<<<1, 1024, 0, st>>>(partial, npartial, out);
    note_launch(2);
    return cuda_status(cudaGetLastError(), "vfwork kernel");
}

// ---------------------------------------------------------------- flux1d test entry
template <typename T>
__global__ void k_flux1d(const T* __restrict__ u, const T* __restrict__ q, T* __restrict__ flux, int nlines, int n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nlines * n) return;
    const int line = (int)(t / n), i = (int)(t % n);
    const T* ql = q + (long long)line * n;
    auto Q = [&](int kk) -> T { return ql[kk]; };
    flux[t] = flux1d_at(i, n, u[t], Q);
}

template <typename T>
int launch_flux1d(const T* u, const T* q, T* flux, int nlines, int n, cudaStream_t st) {
    long long tot = (long long)nlines * n;
    if (tot == 0) return NYLES_OK;
    k_flux1d<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(u, q, flux, nlines, n);
    note_launch();
    return cuda_status(cudaGetLastError(), "flux1d kernel");
}

// ---------------------------------------------------------------- instantiations
#define NYLES_INST(T)                                                                                          \
    template int launch_rhs<T>(const NylesDesc*, const Geom&, const StencilPtrs<T>&, const ProgPtrs<T>&, int, \
                               cudaStream_t, bool, const Bat&);                                                \
    template int launch_update<T>(const Geom&, int, const ProgPtrs<T>&, const ProgPtrs<T>&, const ProgPtrs<T>&, \
                                  const ProgPtrs<T>&, int, double, cudaStream_t, const Bat&);                  \
    template int launch_fill<T>(const Geom&, T* const*, int, cudaStream_t, const Bat&);                        \
    template int launch_diag<T>(const NylesDesc*, const Geom&, const StencilPtrs<T>&, int, cudaStream_t,       \
                                const Bat&);                                                                   \
    template int launch_max_U2<T>(const Geom&, const StencilPtrs<T>&, double*, int, double*, cudaStream_t);   \
    template int launch_vfwork<T>(const Geom&, const StencilPtrs<T>&, const ProgPtrs<T>&, const VfBox&, double*, \
                                  int, double*, cudaStream_t);                                                 \
    template int launch_flux1d<T>(const T*, const T*, T*, int, int, cudaStream_t);
NYLES_INST(double)
NYLES_INST(float)
template int launch_div<double, double>(const NylesDesc*, const Geom&, const StencilPtrs<double>&, double*, cudaStream_t);
template int launch_correct<double, double>(const NylesDesc*, const Geom&, const StencilPtrs<double>&, const double*,
                                            double, cudaStream_t);

// ---------------------------------------------------------------- allocation-free CFL reduction
// The reduction's block partials live in this file-scope array instead of a caller
// workspace. Every GPU that loads the library holds it (8 KiB) until the process exits.
static __device__ __align__(256) double g_static_partials[NYLES_STATIC_PARTIALS];

// Device address of g_static_partials in the current device's context. In host code the
// array's name is only a host-side stand-in; handing it to a kernel would make the
// kernel touch the wrong memory, so only this address is used. The address belongs to
// the context that loaded the module: after cudaDeviceReset (or a primary context that
// a host framework released and re-created) the module loads again, possibly
// elsewhere. So every call made outside stream capture looks the address up afresh
// (a host-side table lookup, no device work) and records it for its device; a call
// made while `st` is capturing uses the address recorded by the last call outside
// capture on that device, and fails with NYLES_BAD_ARG when there is none.
static double* static_partials_for_current_device(cudaStream_t st, int* status) {
    static std::mutex mtx;
    static double* addr[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { *status = cuda_status(e, "cudaGetDevice"); return nullptr; }
    if (dev < 0 || dev >= 64) { set_error("device ordinal above 63"); *status = NYLES_UNSUPPORTED; return nullptr; }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();   // not sticky; treat the stream as capturing
        cs = cudaStreamCaptureStatusActive;
    }
    std::lock_guard<std::mutex> lock(mtx);
    if (cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_partials);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaGetSymbolAddress(g_static_partials)"); return nullptr; }
        addr[dev] = static_cast<double*>(p);
    } else if (!addr[dev]) {
        set_error("max_U2_static: first call on this device made during stream capture; make one call outside "
                  "capture first");
        *status = NYLES_BAD_ARG;
        return nullptr;
    }
    *status = NYLES_OK;
    return addr[dev];
}

}  // namespace nyles

extern "C" int nyles_max_U2_static_f64(const double* U, const double* V, const double* W, long long n,
                                       double* out, void* stream) {
    using namespace nyles;
    if (!U || !V || !W || !out || n <= 0) { set_error("max_U2_static: null array or empty size"); return NYLES_BAD_ARG; }
    if (n > NYLES_STATIC_MAX_CELLS) {
        set_error("max_U2_static: " + std::to_string(n) + " cells exceed the maximum of " +
                  std::to_string((long long)NYLES_STATIC_MAX_CELLS) + " for the static scratch");
        return NYLES_BAD_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int status = NYLES_OK;
    double* partial = static_partials_for_current_device(st, &status);
    if (!partial) return status;
    // one block per 2^18 cells (at least one), at most NYLES_STATIC_PARTIALS blocks
    long long blocks = (n + (1LL << 18) - 1) >> 18;
    if (blocks > NYLES_STATIC_PARTIALS) blocks = NYLES_STATIC_PARTIALS;
    k_max_U2<double><<<(unsigned)blocks, 256, 0, st>>>(n, U, V, W, partial);
    k_max_final<<<1, 1024, 0, st>>>(partial, (int)blocks, out);
    note_launch(2);
    return cuda_status(cudaGetLastError(), "max_U2_static kernel");
}
