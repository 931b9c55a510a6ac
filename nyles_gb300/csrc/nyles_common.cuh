// Shared device code of the Nyles GB300 kernels: array geometry, the WENO3/WENO5
// reconstructions and the 1-D upwind flux with the reference's boundary closures.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef NYLES_MAX_TR
#define NYLES_MAX_TR 8
#endif
#define NYLES_MAX_PROG (4 + NYLES_MAX_TR)
#ifndef NYLES_MAX_BATCH
#define NYLES_MAX_BATCH 32
#endif

namespace nyles {

// ---------------------------------------------------------------- batched launches
// One launch can advance several runs of one bucket (the same grid, precision and
// parameters; each run's fields, registers and workspace in one allocation of the same
// layout). The memory of run r lies `delta[r]` bytes from the memory the kernel's
// arguments point to. A batched kernel's grid repeats the one-run grid along z, once
// per run: the block finds its run from blockIdx.z, shifts every pointer it uses by that
// run's delta and returns at once when the run's gate is closed (the slot holds no run,
// or, inside a multigrid loop, the run's solve has stopped). The table is device
// memory written by the host before each launch (delta, active) and by the multigrid
// control kernels (live, loop_iterations); its layout is NylesBatchTable of the public
// header.
struct BatchTab {
    long long delta[NYLES_MAX_BATCH];
    int active[NYLES_MAX_BATCH];
    int live[NYLES_MAX_BATCH];
    long long loop_iterations;
};
enum { GATE_ACTIVE = 0, GATE_LIVE = 1 };
struct Bat {
    BatchTab* tab = nullptr;   // null: one run, no shift
    int nrun = 1;
    int gate = GATE_ACTIVE;
};

// Run of this block. zb = z-blocks of one run's grid. Returns false when the run is gated
// off; sets bz (the block's z index within its run's grid) and dlt (the byte shift).
__device__ __forceinline__ bool batch_enter(const Bat& b, int& bz, long long& dlt) {
    if (!b.tab) {
        bz = blockIdx.z;
        dlt = 0;
        return true;
    }
    const int zb = gridDim.z / b.nrun;
    const int run = blockIdx.z / zb;
    bz = blockIdx.z - run * zb;
    const int open = b.gate == GATE_LIVE ? b.tab->live[run] : b.tab->active[run];
    dlt = b.tab->delta[run];
    return open != 0;
}
// p shifted by dlt bytes (a null pointer stays null: it marks an unused argument)
template <typename P>
__device__ __forceinline__ P* bshift(P* p, long long dlt) {
    return p ? (P*)((uintptr_t)p + (uintptr_t)dlt) : p;
}

// Model array geometry. Every field is a row-major (z, y, x) array — the layout of the
// reference's `Scalar.view('i')` (core/variables.py:146-151) — with a halo of `nh`
// cells on both sides of each periodic direction and none in closed directions
// (core/mpi/topology.py:253-300). Index 0 = z, 1 = y, 2 = x.
struct Geom {
    int N[3];      // array extents
    int n[3];      // interior extents
    int per[3];    // periodic flags
    int nh;
    long long sz, sy;
    long long vol;

    __host__ __device__ __forceinline__ long long at(int z, int y, int x) const {
        return (long long)z * sz + (long long)y * sy + x;
    }
    __host__ __device__ __forceinline__ long long stride(int d) const {
        return d == 0 ? sz : (d == 1 ? sy : 1);
    }
    // position of the interior cell a halo cell mirrors (periodic self-copy)
    __host__ __device__ __forceinline__ int wrap(int d, int c) const {
        if (!per[d]) return c;
        if (c < nh) return c + n[d];
        if (c >= nh + n[d]) return c - n[d];
        return c;
    }
};

// ---------------------------------------------------------------- WENO constants
// core/weno.f90 keeps REAL(4) literals inside REAL(8) code (f2py build without real
// promotion): each constant is the float value widened to double.
template <typename T> struct WenoK;
template <> struct WenoK<double> {
    static __device__ __forceinline__ double c13() { return (double)(1.0f / 3.0f); }
    static __device__ __forceinline__ double c76() { return (double)(7.0f / 6.0f); }
    static __device__ __forceinline__ double c116() { return (double)(11.0f / 6.0f); }
    static __device__ __forceinline__ double c16() { return (double)(1.0f / 6.0f); }
    static __device__ __forceinline__ double c56() { return (double)(5.0f / 6.0f); }
    static __device__ __forceinline__ double k1() { return (double)(13.0f / 12.0f); }
    static __device__ __forceinline__ double eps5() { return (double)1e-16f; }
    static __device__ __forceinline__ double eps3() { return (double)1e-14f; }
    // `tau5` is implicitly REAL(4) in weno5 (weno.f90:45): round through float
    static __device__ __forceinline__ double tau(double v) { return (double)(float)v; }
};
template <> struct WenoK<float> {
    static __device__ __forceinline__ float c13() { return 1.0f / 3.0f; }
    static __device__ __forceinline__ float c76() { return 7.0f / 6.0f; }
    static __device__ __forceinline__ float c116() { return 11.0f / 6.0f; }
    static __device__ __forceinline__ float c16() { return 1.0f / 6.0f; }
    static __device__ __forceinline__ float c56() { return 5.0f / 6.0f; }
    static __device__ __forceinline__ float k1() { return 13.0f / 12.0f; }
    static __device__ __forceinline__ float eps5() { return 1e-16f; }
    static __device__ __forceinline__ float eps3() { return 1e-14f; }
    static __device__ __forceinline__ float tau(float v) { return v; }
};

// core/weno.f90:1-22
template <typename T>
__device__ __forceinline__ T weno3(T qm, T q0, T qp) {
    typedef WenoK<T> K;
    T qi1 = (-qm + T(3) * q0) * T(0.5);
    T qi2 = (q0 + qp) * T(0.5);
    T d1 = q0 - qm, d2 = qp - q0;
    T beta1 = d1 * d1, beta2 = d2 * d2;
    T tau = fabs(beta2 - beta1);
    T w1 = T(1) + tau / (beta1 + K::eps3());
    T w2 = (T(1) + tau / (beta2 + K::eps3())) * T(2);
    return (w1 * qi1 + w2 * qi2) / (w1 + w2);
}

// core/weno.f90:25-54
template <typename T>
__device__ __forceinline__ T weno5(T qmm, T qm, T q0, T qp, T qpp) {
    typedef WenoK<T> K;
    T qi1 = K::c13() * qmm - K::c76() * qm + K::c116() * q0;
    T qi2 = -(K::c16() * qm) + K::c56() * q0 + K::c13() * qp;
    T qi3 = K::c13() * q0 + K::c56() * qp - K::c16() * qpp;
    T a1 = qmm - T(2) * qm + q0, b1 = qmm - T(4) * qm + T(3) * q0;
    T a2 = qm - T(2) * q0 + qp, b2 = qm - qp;
    T a3 = q0 - T(2) * qp + qpp, b3 = T(3) * q0 - T(4) * qp + qpp;
    T beta1 = K::k1() * (a1 * a1) + T(0.25) * (b1 * b1);
    T beta2 = K::k1() * (a2 * a2) + T(0.25) * (b2 * b2);
    T beta3 = K::k1() * (a3 * a3) + T(0.25) * (b3 * b3);
    T tau5 = K::tau(fabs(beta1 - beta3));
    T w1 = T(1) + tau5 / (beta1 + K::eps5());
    T w2 = T(6) * (T(1) + tau5 / (beta2 + K::eps5()));
    T w3 = T(3) * (T(1) + tau5 / (beta3 + K::eps5()));
    return (w1 * qi1 + w2 * qi2 + w3 * qi3) / (w1 + w2 + w3);
}

// Double precision: the same reconstruction with one division instead of four.
// With d_k = beta_k + eps and e_k = d_k + tau5, the weights are w1 = e1/d1,
// w2 = 6 e2/d2, w3 = 3 e3/d3; multiplying numerator and denominator of
// sum(w_k qi_k)/sum(w_k) by d1 d2 d3 leaves positive terms only, so the result
// differs from the four-division form by rounding alone. d_k >= 1e-16 keeps the
// triple products far from underflow in double (not so in float, which keeps the
// form above). FP64 division is a multi-instruction sequence on the FP64 pipe, the
// scarce unit on GB300.
template <>
__device__ __forceinline__ double weno5<double>(double qmm, double qm, double q0, double qp, double qpp) {
    typedef WenoK<double> K;
    const double qi1 = K::c13() * qmm - K::c76() * qm + K::c116() * q0;
    const double qi2 = -(K::c16() * qm) + K::c56() * q0 + K::c13() * qp;
    const double qi3 = K::c13() * q0 + K::c56() * qp - K::c16() * qpp;
    const double a1 = qmm - 2.0 * qm + q0, b1 = qmm - 4.0 * qm + 3.0 * q0;
    const double a2 = qm - 2.0 * q0 + qp, b2 = qm - qp;
    const double a3 = q0 - 2.0 * qp + qpp, b3 = 3.0 * q0 - 4.0 * qp + qpp;
    const double beta1 = K::k1() * (a1 * a1) + 0.25 * (b1 * b1);
    const double beta2 = K::k1() * (a2 * a2) + 0.25 * (b2 * b2);
    const double beta3 = K::k1() * (a3 * a3) + 0.25 * (b3 * b3);
    const double tau5 = K::tau(fabs(beta1 - beta3));
    const double d1 = beta1 + K::eps5(), d2 = beta2 + K::eps5(), d3 = beta3 + K::eps5();
    const double A = (d1 + tau5) * (d2 * d3);
    const double B = 6.0 * (d2 + tau5) * (d1 * d3);
    const double C = 3.0 * (d3 + tau5) * (d1 * d2);
    return (A * qi1 + B * qi2 + C * qi3) / (A + B + C);
}

// Single precision (mixed-precision path): the four-division form with the hardware
// reciprocal-based division (__fdividef, within 2 ulp): every denominator here is at
// least 1e-14 or 1e-16 (eps) and far below 2^126, the limit of its accurate range, and
// the weights only scale the stencils.
template <>
__device__ __forceinline__ float weno3<float>(float qm, float q0, float qp) {
    typedef WenoK<float> K;
    const float qi1 = (-qm + 3.f * q0) * 0.5f;
    const float qi2 = (q0 + qp) * 0.5f;
    const float d1 = q0 - qm, d2 = qp - q0;
    const float beta1 = d1 * d1, beta2 = d2 * d2;
    const float tau = fabsf(beta2 - beta1);
    const float w1 = 1.f + __fdividef(tau, beta1 + K::eps3());
    const float w2 = (1.f + __fdividef(tau, beta2 + K::eps3())) * 2.f;
    return __fdividef(w1 * qi1 + w2 * qi2, w1 + w2);
}
template <>
__device__ __forceinline__ float weno5<float>(float qmm, float qm, float q0, float qp, float qpp) {
    typedef WenoK<float> K;
    const float qi1 = K::c13() * qmm - K::c76() * qm + K::c116() * q0;
    const float qi2 = -(K::c16() * qm) + K::c56() * q0 + K::c13() * qp;
    const float qi3 = K::c13() * q0 + K::c56() * qp - K::c16() * qpp;
    const float a1 = qmm - 2.f * qm + q0, b1 = qmm - 4.f * qm + 3.f * q0;
    const float a2 = qm - 2.f * q0 + qp, b2 = qm - qp;
    const float a3 = q0 - 2.f * qp + qpp, b3 = 3.f * q0 - 4.f * qp + qpp;
    const float beta1 = K::k1() * (a1 * a1) + 0.25f * (b1 * b1);
    const float beta2 = K::k1() * (a2 * a2) + 0.25f * (b2 * b2);
    const float beta3 = K::k1() * (a3 * a3) + 0.25f * (b3 * b3);
    const float tau5 = fabsf(beta1 - beta3);
    const float w1 = 1.f + __fdividef(tau5, beta1 + K::eps5());
    const float w2 = 6.f * (1.f + __fdividef(tau5, beta2 + K::eps5()));
    const float w3 = 3.f * (1.f + __fdividef(tau5, beta3 + K::eps5()));
    return __fdividef(w1 * qi1 + w2 * qi2 + w3 * qi3, w1 + w2 + w3);
}

// Value of core/weno.f90:106-153 `flux1d` at index i (0-based) of a line of length n
// (n >= 5), given the velocity u at i and an accessor Q(j) for the advected quantity.
// Branch precedence follows the Fortran statement order (later statements win).
// In the interior the five stencil values are selected by the sign of u before a
// single weno5 evaluation, so lanes of a warp do not diverge on the upwind side.
template <typename T, typename QF>
__device__ __forceinline__ T flux1d_at(int i, int n, T u, QF Q) {
    if (i >= 2 && i <= n - 4) {
        bool pos = u > T(0);
        T qa = pos ? Q(i - 2) : Q(i + 3);
        T qb = pos ? Q(i - 1) : Q(i + 2);
        T qc = pos ? Q(i) : Q(i + 1);
        T qd = pos ? Q(i + 1) : Q(i);
        T qe = pos ? Q(i + 2) : Q(i - 1);
        return u * weno5(qa, qb, qc, qd, qe);
    }
    if (i == n - 1) return T(0);
    if (i == n - 2) return (u > T(0)) ? u * weno3(Q(i - 1), Q(i), Q(i + 1)) : u * Q(i + 1);
    if (i == n - 3)
        return (u > T(0)) ? u * weno5(Q(i - 2), Q(i - 1), Q(i), Q(i + 1), Q(i + 2))
                          : u * weno3(Q(i + 2), Q(i + 1), Q(i));
    if (i == 1) return (u > T(0)) ? u * weno3(Q(0), Q(1), Q(2)) : u * weno5(Q(4), Q(3), Q(2), Q(1), Q(0));
    return (u > T(0)) ? u * Q(0) : u * weno3(Q(2), Q(1), Q(0));
}

// ---------------------------------------------------------------- exact rounding
// Operations that must round once each, as numpy and gfortran do (no fused multiply-
// add): elementwise time-scheme updates, differences and metric products.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// ---------------------------------------------------------------- float pairs
// A value carried as hi + lo, two floats with |lo| <= ulp(hi)/2 (about 48 significant
// bits), built from error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum
// (|a| >= |b|) and the FMA-based TwoProduct. The mixed-precision projection keeps its
// solution and right-hand side in this form, so that the extended-precision residual
// and correction of iterative refinement run on the FP32 pipes (GB300 issues FP64
// instructions at a small fraction of the FP32 rate). Every step rounds once
// (explicit _rn intrinsics), so no contraction can break the error terms.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}
// (a.hi + a.lo) + b, renormalised
__device__ __forceinline__ float2 df_add_f(float2 a, float b) {
    float s, e;
    two_sum(a.x, b, s, e);
    e = __fadd_rn(e, a.y);
    float2 r;
    fast_two_sum(s, e, r.x, r.y);
    return r;
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float s, e;
    two_sum(a.x, b.x, s, e);
    e = __fadd_rn(e, __fadd_rn(a.y, b.y));
    float2 r;
    fast_two_sum(s, e, r.x, r.y);
    return r;
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
// u * (c.hi + c.lo) for a float u
__device__ __forceinline__ float2 df_mul_f(float u, float2 c) {
    float p, e;
    two_prod(u, c.x, p, e);
    e = __fmaf_rn(u, c.y, e);
    float2 r;
    fast_two_sum(p, e, r.x, r.y);
    return r;
}
// (a.hi + a.lo) * (c.hi + c.lo)
__device__ __forceinline__ float2 df_mul(float2 a, float2 c) {
    float p, e;
    two_prod(a.x, c.x, p, e);
    e = __fmaf_rn(a.x, c.y, e);
    e = __fmaf_rn(a.y, c.x, e);
    float2 r;
    fast_two_sum(p, e, r.x, r.y);
    return r;
}
__device__ __forceinline__ float df_value(float2 a) { return __fadd_rn(a.x, a.y); }
// host: split a double into a float pair
inline float2 df_split(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

// ---------------------------------------------------------------- reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace nyles
