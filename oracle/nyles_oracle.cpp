// CPU ORACLE — test infrastructure only.
//
// A C++ restatement of the Nyles LES time step (pvthinker/Nyles),
// used by the test-suite and by bench.py's CPU-baseline leg as the checker of the
// CUDA path. It is never linked into, called by, or shipped with the product library.
//
// Parity status: the reference's Fortran kernels cannot be compiled in this
// environment (no Fortran compiler), so the kernel restatements below are checked by
// known-answer tests taken from the reference's own __main__ demos plus analytic
// properties. The orchestration (views, halo fills, projection glue, time schemes)
// is pinned against the reference's own Python modules, imported with this file's
// kernels standing in for the f2py/ctypes libraries (tests/golden/make_golden.py).
// Kernel-level parity is therefore "partially pinned". Two branches have no reference
// output to pin against at all ("parity unpinned"): the linear tracer schemes
// (upwind_linear, interpolate_tracer: the reference hard-codes WENO) and the advection
// model (the reference's constructor cannot run); their restatements are checked by a
// numpy restatement, convergence orders and conservation (tests/test_advection.py).
//
// Arithmetic follows the Fortran source operation by operation (association order,
// REAL(4) literals and the implicitly REAL(4) `tau5` of weno5). Compile with
// -ffp-contract=off so that no fused multiply-add changes the rounding.
//
// Layout: every model field is a C-order array of shape (Nz, Ny, Nx) — the
// reference's `view('i')` — including halos in periodic directions. The reference's
// transposed views are expressed as strided views of that one array.
//
// Threads: the outer loop of each stencil and multigrid sweep may be split into
// contiguous chunks run on several host threads (orc_set_threads; the environment
// variable NYLES_ORACLE_THREADS, default 1). Every element is still computed by the
// same expression from the same inputs and no two chunks write the same element; the
// sums (multigrid norms, VFwork) stay sequential. Results are therefore identical for
// every thread count.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <string>
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <thread>

namespace {

// ---------------------------------------------------------------- host threads
std::atomic<int> g_threads{0};   // 0: not read yet

int oracle_threads() {
    int n = g_threads.load();
    if (n == 0) {
        const char* e = std::getenv("NYLES_ORACLE_THREADS");
        n = e ? std::atoi(e) : 1;
        if (n <= 0) n = (int)std::thread::hardware_concurrency();
        n = std::max(1, std::min(n, 256));
        g_threads.store(n);
    }
    return n;
}

// f(lo, hi) over [0, n) in contiguous chunks, one per thread, when the loop does at
// least 2^16 elements of work in total (`work` per index); inline otherwise
template <class F>
void pfor(int n, long work, F&& f) {
    int nt = std::min(oracle_threads(), n);
    if (nt <= 1 || (long)n * work < (1L << 16)) {
        if (n > 0) f(0, n);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (int t = 1; t < nt; ++t)
        th.emplace_back([&f, n, nt, t] { f((int)((long)n * t / nt), (int)((long)n * (t + 1) / nt)); });
    f(0, (int)((long)n / nt));
    for (auto& x : th) x.join();
}

// elementwise loops over [0, vol) in 4096-element blocks
template <class F>
void pfor_elems(long vol, F&& f) {
    const long blk = 4096;
    const int nb = (int)((vol + blk - 1) / blk);
    pfor(nb, blk, [&](int b0, int b1) {
        const long c0 = (long)b0 * blk, c1 = std::min(vol, (long)b1 * blk);
        for (long c = c0; c < c1; ++c) f(c);
    });
}

// ---------------------------------------------------------------- strided views
struct V3 {
    double* p;
    int n0, n1, n2;     // extents in the view's index order (Fortran dims l,m,n)
    long s0, s1, s2;    // strides in elements
    inline double& operator()(int a, int b, int c) const { return p[a * s0 + b * s1 + c * s2]; }
};

// logical field (z,y,x) C-order, extents N[0]=Nz, N[1]=Ny, N[2]=Nx
// view('i') = (z,y,x), view('j') = (x,z,y), view('k') = (y,x,z)   core/variables.py:162-182
V3 view(double* p, const int N[3], char d) {
    long sz = (long)N[1] * N[2], sy = N[2], sx = 1;
    switch (d) {
        case 'i': return V3{p, N[0], N[1], N[2], sz, sy, sx};
        case 'j': return V3{p, N[2], N[0], N[1], sx, sz, sy};
        default:  return V3{p, N[1], N[2], N[0], sy, sx, sz};
    }
}
// flipview: direction d outermost   core/variables.py:184-204
V3 flipview(double* p, const int N[3], char d) {
    return view(p, N, d == 'i' ? 'j' : (d == 'j' ? 'k' : 'i'));
}

// ---------------------------------------------------------------- WENO   core/weno.f90
// REAL(4) literal constants promoted to REAL(8) at use (f2py build, no real promotion).
const double W5_C13 = (double)(1.0f / 3.0f);
const double W5_C76 = (double)(7.0f / 6.0f);
const double W5_C116 = (double)(11.0f / 6.0f);
const double W5_C16 = (double)(1.0f / 6.0f);
const double W5_C56 = (double)(5.0f / 6.0f);
const double W5_K1 = (double)(13.0f / 12.0f);
const double W5_EPS = (double)1e-16f;
const double W3_EPS = (double)1e-14f;

// core/weno.f90:1-22
double weno3(double qm, double q0, double qp) {
    double qi1 = (-qm + 3.0 * q0) * 0.5;
    double qi2 = (q0 + qp) * 0.5;
    double d1 = q0 - qm, d2 = qp - q0;
    double beta1 = d1 * d1;
    double beta2 = d2 * d2;
    double tau = std::fabs(beta2 - beta1);
    double w1 = 1.0 + tau / (beta1 + W3_EPS);
    double w2 = (1.0 + tau / (beta2 + W3_EPS)) * 2.0;
    return (w1 * qi1 + w2 * qi2) / (w1 + w2);
}

// core/weno.f90:25-54 ; `tau5` is implicitly REAL(4) (no implicit none, weno.f90:45)
double weno5(double qmm, double qm, double q0, double qp, double qpp) {
    double qi1 = W5_C13 * qmm - W5_C76 * qm + W5_C116 * q0;
    double qi2 = -(W5_C16 * qm) + W5_C56 * q0 + W5_C13 * qp;
    double qi3 = W5_C13 * q0 + W5_C56 * qp - W5_C16 * qpp;
    double a1 = qmm - 2.0 * qm + q0, b1 = qmm - 4.0 * qm + 3.0 * q0;
    double a2 = qm - 2.0 * q0 + qp, b2 = qm - qp;
    double a3 = q0 - 2.0 * qp + qpp, b3 = 3.0 * q0 - 4.0 * qp + qpp;
    double beta1 = W5_K1 * (a1 * a1) + 0.25 * (b1 * b1);
    double beta2 = W5_K1 * (a2 * a2) + 0.25 * (b2 * b2);
    double beta3 = W5_K1 * (a3 * a3) + 0.25 * (b3 * b3);
    float tau5f = (float)std::fabs(beta1 - beta3);
    double tau5 = (double)tau5f;
    double w1 = 1.0 + tau5 / (beta1 + W5_EPS);
    double w2 = 6.0 * (1.0 + tau5 / (beta2 + W5_EPS));
    double w3 = 3.0 * (1.0 + tau5 / (beta3 + W5_EPS));
    return (w1 * qi1 + w2 * qi2 + w3 * qi3) / (w1 + w2 + w3);
}

// core/weno.f90:106-153 (0-based here: index i of the Fortran routine is i-1)
// Assignment order of the Fortran routine is kept so that for short lines later
// statements overwrite earlier ones exactly as in the reference.
void flux1d(const double* u, const double* q, double* flux, int n) {
    // i = 1
    flux[0] = (u[0] > 0) ? u[0] * q[0] : u[0] * weno3(q[2], q[1], q[0]);
    // i = 2
    flux[1] = (u[1] > 0) ? u[1] * weno3(q[0], q[1], q[2]) : u[1] * weno5(q[4], q[3], q[2], q[1], q[0]);
    // i = 3 .. n-3
    for (int i = 2; i <= n - 4; ++i) {
        if (u[i] > 0) flux[i] = u[i] * weno5(q[i - 2], q[i - 1], q[i], q[i + 1], q[i + 2]);
        else          flux[i] = u[i] * weno5(q[i + 3], q[i + 2], q[i + 1], q[i], q[i - 1]);
    }
    // i = n-2
    { int i = n - 3;
      if (u[i] > 0) flux[i] = u[i] * weno5(q[i - 2], q[i - 1], q[i], q[i + 1], q[i + 2]);
      else          flux[i] = u[i] * weno3(q[i + 2], q[i + 1], q[i]); }
    // i = n-1
    { int i = n - 2;
      if (u[i] > 0) flux[i] = u[i] * weno3(q[i - 1], q[i], q[i + 1]);
      else          flux[i] = u[i] * q[i + 1]; }
    flux[n - 1] = 0.0;
}

// ---------------------------------------------------------------- vortex force
// core/fortran_vortex_force.f90:10-85 (WENO branch; `linear` is hard-wired .false.)
// arrays in (j, i, k) convention, dims (m, n, l)
void vortex_force_direc(const V3& U, const V3& vort, const V3& res) {
    const int m = U.n0, n = U.n1, l = U.n2;
    pfor(m, (long)n * l, [&](int j0, int j1) {
    std::vector<double> u1d(l), q(l), flux(l);
    for (int j = j0; j < j1; ++j) {
        for (int i = 0; i < n - 1; ++i) {
            double UU_0 = 0.0;
            for (int k = 0; k < l; ++k) {
                double UU_1 = 0.5 * (U(j, i, k) + U(j, i + 1, k));
                u1d[k] = 0.5 * (UU_0 + UU_1);
                UU_0 = UU_1;
            }
            q[0] = 0.0;
            for (int k = 1; k < l; ++k) q[k] = vort(j, i, k - 1);
            flux1d(u1d.data(), q.data(), flux.data(), l);
            for (int k = 0; k < l; ++k) res(j, i, k) = res(j, i, k) - flux[k];
        }
    }
    });
}

// core/fortran_vortex_force.f90:87-165 (WENO branch)
void vortex_force_flip(const V3& U, const V3& vort, const V3& res) {
    const int m = U.n0, n = U.n1, l = U.n2;
    pfor(m, (long)n * l, [&](int j0, int j1) {
    std::vector<double> u1d(n), q(n), flux(n);
    for (int j = j0; j < j1; ++j) {
        for (int k = 0; k < l - 1; ++k) {
            double UU_0 = 0.0;
            for (int i = 0; i < n; ++i) {
                double UU_1 = 0.5 * (U(j, i, k) + U(j, i, k + 1));
                u1d[i] = 0.5 * (UU_0 + UU_1);
                UU_0 = UU_1;
            }
            q[0] = 0.0;
            for (int i = 1; i < n; ++i) q[i] = vort(j, i - 1, k);
            flux1d(u1d.data(), q.data(), flux.data(), n);
            for (int i = 0; i < n; ++i) res(j, i, k) = res(j, i, k) + flux[i];
        }
    }
    });
}

// core/interpolate.f90:3-112 (the vortex-force interpolation) in its own 1-based
// indexing: vU[1..n], qp[0..n-1], qm[1..n] (index 0 of vU and qm unused). The
// coefficients are REAL(4) literals widened to double. Entries the Fortran leaves
// unset are left as they are (never read by the callers).
void interpolate_vf(const double* vU, double* qp, double* qm, int order, int n) {
    const double c1 = (double)(-1.0f / 6.0f), c2 = (double)(5.0f / 6.0f), c3 = (double)(2.0f / 6.0f);
    const double e1 = (double)(-1.0f / 12.0f), e2 = (double)(7.0f / 12.0f);
    const double b1 = (double)(2.0f / 60.0f), b2 = (double)(-13.0f / 60.0f), b3 = (double)(47.0f / 60.0f),
                 b4 = (double)(27.0f / 60.0f), b5 = (double)(-3.0f / 60.0f);
    int i;
    if (order == 5) {
        qp[0] = 0.0;
        i = 1; qp[i] = vU[i]; qm[i] = vU[i];
        i = 2;
        qp[i] = c1 * vU[i - 1] + c2 * vU[i] + c3 * vU[i + 1];
        qm[i] = c3 * vU[i - 1] + c2 * vU[i] + c1 * vU[i + 1];
        for (i = 3; i <= n - 3; ++i) {
            qp[i] = b1 * vU[i - 2] + b2 * vU[i - 1] + b3 * vU[i] + b4 * vU[i + 1] + b5 * vU[i + 2];
            qm[i] = b5 * vU[i - 2] + b4 * vU[i - 1] + b3 * vU[i] + b2 * vU[i + 1] + b1 * vU[i + 2];
        }
        i = n - 2;
        qp[i] = c1 * vU[i - 1] + c2 * vU[i] + c3 * vU[i + 1];
        qm[i] = c3 * vU[i - 1] + c2 * vU[i] + c1 * vU[i + 1];
        i = n - 1; qp[i] = vU[i]; qm[i] = vU[i];
        qm[n] = vU[n];
    } else if (order == 3) {
        qp[0] = 0.0;
        i = 1; qp[i] = vU[i]; qm[i] = vU[i];
        for (i = 2; i <= n - 2; ++i) {
            qp[i] = c1 * vU[i - 1] + c2 * vU[i] + c3 * vU[i + 1];
            qm[i] = c3 * vU[i - 1] + c2 * vU[i] + c1 * vU[i + 1];
        }
        i = n - 1; qp[i] = vU[i]; qm[i] = vU[i];
        qm[n] = vU[n];
    } else if (order == 1) {
        qp[0] = 0.0;
        for (i = 1; i <= n - 1; ++i) { qp[i] = vU[i]; qm[i] = vU[i]; }
        qm[n] = vU[n];
    } else if (order == 2) {
        qm[1] = 0.5 * vU[1];
        for (i = 2; i <= n; ++i) qm[i] = 0.5 * (vU[i - 1] + vU[i]);
    } else if (order == 4) {
        i = 1; qm[i] = e2 * (vU[i]) + e1 * (vU[i + 1]);
        i = 2; qm[i] = e2 * (vU[i - 1] + vU[i]) + e1 * (vU[i + 1]);
        for (i = 3; i <= n - 1; ++i) qm[i] = e2 * (vU[i - 1] + vU[i]) + e1 * (vU[i - 2] + vU[i + 1]);
        i = n; qm[i] = e2 * (vU[i - 1] + vU[i]) + e1 * (vU[i - 2]);
    }
}

// core/fortran_vortex_force.f90:43-55 (direc) and :121-133 (flip), the linear branch the
// reference never takes (`linear = .false.`): the vorticity of the line, unshifted, is
// interpolated with core/interpolate.f90 of order `order`; odd orders upwind qp/qm with
// the positive/negative parts of the doubly averaged velocity, even orders add the
// interpolated vorticity alone (as written there). `sign` = -1 for direc, +1 for flip;
// the two products are applied one after the other, in the Fortran statement order.
void vf_linear_line(const double* U0, const double* U1, long su, const double* vort, long sv, double* res, long sr,
                    int len, int order, int sign, std::vector<double>& vU, std::vector<double>& qp,
                    std::vector<double>& qm, std::vector<double>& up, std::vector<double>& um) {
    double UU_0 = 0.0;
    for (int k = 1; k <= len; ++k) {
        double UU_1 = 0.5 * (U0[(k - 1) * su] + U1[(k - 1) * su]);
        vU[k] = vort[(k - 1) * sv];
        double Ui = 0.5 * (UU_0 + UU_1);
        double UU = std::fabs(Ui);
        up[k] = 0.5 * (Ui + UU);
        um[k] = 0.5 * (Ui - UU);
        UU_0 = UU_1;
    }
    interpolate_vf(vU.data(), qp.data(), qm.data(), order, len);
    for (int k = 1; k <= len; ++k) {
        double& r = res[(k - 1) * sr];
        if (order % 2 == 0) r = (sign < 0) ? r - qm[k] : r + qm[k];
        else r = (sign < 0) ? r - qp[k - 1] * up[k] - qm[k] * um[k] : r + qp[k - 1] * up[k] + qm[k] * um[k];
    }
}

void vortex_force_direc_linear(const V3& U, const V3& vort, const V3& res, int order) {
    const int m = U.n0, n = U.n1, l = U.n2;
    pfor(m, (long)n * l, [&](int j0, int j1) {
    std::vector<double> vU(l + 1), qp(l + 1, 0.0), qm(l + 1, 0.0), up(l + 1), um(l + 1);
    for (int j = j0; j < j1; ++j)
        for (int i = 0; i < n - 1; ++i)
            vf_linear_line(&U(j, i, 0), &U(j, i + 1, 0), U.s2, &vort(j, i, 0), vort.s2, &res(j, i, 0), res.s2, l,
                           order, -1, vU, qp, qm, up, um);
    });
}

void vortex_force_flip_linear(const V3& U, const V3& vort, const V3& res, int order) {
    const int m = U.n0, n = U.n1, l = U.n2;
    pfor(m, (long)n * l, [&](int j0, int j1) {
    std::vector<double> vU(n + 1), qp(n + 1, 0.0), qm(n + 1, 0.0), up(n + 1), um(n + 1);
    for (int j = j0; j < j1; ++j)
        for (int k = 0; k < l - 1; ++k)
            vf_linear_line(&U(j, 0, k), &U(j, 0, k + 1), U.s1, &vort(j, 0, k), vort.s1, &res(j, 0, k), res.s1, n,
                           order, +1, vU, qp, qm, up, um);
    });
}

// ---------------------------------------------------------------- tracer flux
// core/fortran_upwind.f90:3-87 (WENO branch), dims (l, m, n), direction = last index
void upwind(const V3& trac, const V3& u, const V3& dtrac) {
    const int l = trac.n0, m = trac.n1, n = trac.n2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    std::vector<double> up(n), phi(n), flux(n);
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j) {
            for (int i = 0; i < n; ++i) { up[i] = u(k, j, i); phi[i] = trac(k, j, i); }
            flux1d(up.data(), phi.data(), flux.data(), n);
            dtrac(k, j, 0) = dtrac(k, j, 0) - flux[0];
            for (int i = 1; i < n; ++i) dtrac(k, j, i) = dtrac(k, j, i) + flux[i - 1] - flux[i];
        }
    });
}

// core/interpolate_tracer.f90:3-116 on one line of n values (0-based here; the source is
// 1-based). The coefficients are REAL(4) literals widened to double.
void interpolate_tracer(const double* q, double* qp, double* qm, int order, int n) {
    const double c1 = -1.0f / 6.0f, c2 = 5.0f / 6.0f, c3 = 2.0f / 6.0f;
    const double e1 = -1.0f / 12.0f, e2 = 7.0f / 12.0f;
    const double b1 = 2.0f / 60.0f, b2 = -13.0f / 60.0f, b3 = 47.0f / 60.0f, b4 = 27.0f / 60.0f,
                 b5 = -3.0f / 60.0f;
    auto cstencil = [&](int i) {
        qp[i] = c1 * q[i - 1] + c2 * q[i] + c3 * q[i + 1];
        qm[i] = c3 * q[i - 1] + c2 * q[i] + c1 * q[i + 1];
    };
    if (order == 5) {
        qp[0] = q[0]; qm[0] = q[0];
        cstencil(1);
        for (int i = 2; i <= n - 3; ++i) {
            qp[i] = b1 * q[i - 2] + b2 * q[i - 1] + b3 * q[i] + b4 * q[i + 1] + b5 * q[i + 2];
            qm[i] = b5 * q[i - 2] + b4 * q[i - 1] + b3 * q[i] + b2 * q[i + 1] + b1 * q[i + 2];
        }
        cstencil(n - 2);
        qp[n - 1] = q[n - 1]; qm[n - 1] = q[n - 1];
    } else if (order == 3) {
        qp[0] = q[0]; qm[0] = q[0];
        for (int i = 1; i <= n - 2; ++i) cstencil(i);
        qp[n - 1] = q[n - 1]; qm[n - 1] = q[n - 1];
    } else if (order == 1) {
        for (int i = 0; i < n; ++i) { qp[i] = q[i]; qm[i] = q[i]; }
    } else if (order == 2) {
        for (int i = 0; i < n - 1; ++i) qp[i] = 0.5 * (q[i] + q[i + 1]);
    } else if (order == 4) {
        qp[0] = e2 * (q[0] + q[1]) + e1 * (q[2]);
        for (int i = 1; i <= n - 3; ++i) qp[i] = e2 * (q[i] + q[i + 1]) + e1 * (q[i - 1] + q[i + 2]);
        qp[n - 2] = e2 * (q[n - 2] + q[n - 1]) + e1 * (q[n - 3]);
    }
}

// core/fortran_upwind.f90:32-61, the linear branch (`linear` is .false. in the
// reference, so only an explicit order > 0 reaches it): odd orders upwind the
// interpolations qp(i) / qm(i+1) with the split velocity, even orders take the centred
// qp(i); the last face carries no flux.
void upwind_linear(const V3& trac, const V3& u, const V3& dtrac, int order) {
    const int l = trac.n0, m = trac.n1, n = trac.n2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    std::vector<double> up(n), um(n), phi(n), qp(n, 0.0), qm(n, 0.0);
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j) {
            for (int i = 0; i < n; ++i) {
                double uu = std::fabs(u(k, j, i));
                up[i] = 0.5 * (u(k, j, i) + uu);
                um[i] = 0.5 * (u(k, j, i) - uu);
                phi[i] = trac(k, j, i);
            }
            interpolate_tracer(phi.data(), qp.data(), qm.data(), order, n);
            double fxm = 0.0, fx;
            for (int i = 0; i < n - 1; ++i) {
                fx = (order % 2 == 0) ? u(k, j, i) * qp[i] : up[i] * qp[i] + um[i] * qm[i + 1];
                dtrac(k, j, i) = dtrac(k, j, i) + fxm - fx;
                fxm = fx;
            }
            fx = 0.0;
            dtrac(k, j, n - 1) = dtrac(k, j, n - 1) + fxm - fx;
        }
    });
}

// ---------------------------------------------------------------- vorticity
// core/fortran_vorticity.f90:2-28
void vorticity_k(const V3& ui, const V3& uj, const V3& wk) {
    const int l = ui.n0, m = ui.n1, n = ui.n2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m - 1; ++j) {
            for (int i = 0; i < n - 1; ++i)
                wk(k, j, i) = uj(k, j, i + 1) - uj(k, j, i) - ui(k, j + 1, i) + ui(k, j, i);
            wk(k, j, n - 1) = 0.0;
        }
    });
}

// ---------------------------------------------------------------- kinetic energy
// core/fortran_kinenergy.f90:3-56
void kin(const V3& u, const V3& ke, double ds2) {
    const int l = u.n0, m = u.n1, n = u.n2;
    double cff2 = 0.5 * ds2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j)
            for (int i = 1; i < n; ++i) {
                double a = u(k, j, i), b = u(k, j, i - 1);
                ke(k, j, i) = ke(k, j, i) + cff2 * 0.5 * (a * a + b * b);
            }
    });
}

// ---------------------------------------------------------------- Bernoulli / div
// core/fortran_bernoulli.f90:2-26
void gradke(const V3& ke, const V3& du) {
    const int l = ke.n0, m = ke.n1, n = ke.n2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n - 1; ++i)
                du(k, j, i) = du(k, j, i) - (ke(k, j, i + 1) - ke(k, j, i));
    });
}
// core/fortran_bernoulli.f90:29-58
void gradkeandb(const V3& ke, const V3& b, const V3& du, double dz) {
    const int l = ke.n0, m = ke.n1, n = ke.n2;
    double cff = 0.5 * dz;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n - 1; ++i)
                du(k, j, i) = du(k, j, i) - (ke(k, j, i + 1) - ke(k, j, i)) + cff * (b(k, j, i + 1) + b(k, j, i));
    });
}
// core/fortran_bernoulli.f90:61-97
void divop(const V3& d, const V3& u, int iflag) {
    const int l = d.n0, m = d.n1, n = d.n2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j) {
            if (iflag > 0) {
                d(k, j, 0) = d(k, j, 0) + u(k, j, 0);
                for (int i = 1; i < n; ++i) d(k, j, i) = d(k, j, i) + (u(k, j, i) - u(k, j, i - 1));
            } else {
                d(k, j, 0) = u(k, j, 0);
                for (int i = 1; i < n; ++i) d(k, j, i) = (u(k, j, i) - u(k, j, i - 1));
            }
        }
    });
}
// core/fortran_dissipation.f90:2-35
void add_laplacian(const V3& phi, const V3& dphi, double coef) {
    const int l = phi.n0, m = phi.n1, n = phi.n2;
    pfor(l, (long)m * n, [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < m; ++j) {
            double fxm = 0.0, fx;
            for (int i = 0; i < n - 1; ++i) {
                fx = phi(k, j, i + 1) - phi(k, j, i);
                dphi(k, j, i) = dphi(k, j, i) + coef * (fx - fxm);
                fxm = fx;
            }
            fx = 0.0;
            dphi(k, j, n - 1) = dphi(k, j, n - 1) + coef * (fx - fxm);
        }
    });
}

V3 contig(double* p, int l, int m, int n) { return V3{p, l, m, n, (long)m * n, n, 1}; }

// ================================================================ multigrid (mgfor)
// Restatement of core/mgfor for one rank (npx = npy = 1), cell-centred 3-D path.
// Arrays are Fortran (i, j, k) with i in [1-nh, nx+nh], j in [1-nh, ny+nh],
// k in [1, nz] where nz already includes 2*nh ghost layers (mg_setup.f90:15-35,
// mg_setup.f90:225-307). Storage: i fastest.
enum { CLOSED = 1, XPERIO, YPERIO, ZPERIO, XYPERIO, XYZPERIO };   // mg_enums.f90:6

struct MgLevel {
    int nx, ny, nz, nh;
    long pi, pj;   // strides
    std::vector<double> x, b, r, y, diag, idiag, Rcoef, Pcoef;
    std::vector<int> msk;
    long at(int i, int j, int k) const { return (long)(i + nh - 1) + pi * (j + nh - 1) + pj * (k - 1); }
    long size() const { return (long)(nx + 2 * nh) * (ny + 2 * nh) * nz; }
};

struct Mg {
    int nlevels = 0, nh = 3, topology = CLOSED;
    // MG_Param defaults (mg_types.f90:15-26); the multigrid category of
    // defaults.json is never passed to mgfor (core/mgfordriver.py:24).
    int maxite = 20;
    double tol = 1e-6, omega = 0.9;
    int nite = 0;
    double res = 0.0;
    bool xper = false, yper = false, zper = false;
    std::vector<MgLevel> L;   // index 0 = level 1
};

// mod_halo.f90:235-262 (exchange_with_myself). Fortran array assignment semantics:
// the right-hand side is evaluated before any element is stored.
void mg_fill(const Mg& mg, const MgLevel& g, double* a) {
    const int nx = g.nx, ny = g.ny, nz = g.nz, nh = g.nh;
    auto A = [&](int i, int j, int k) -> double& { return a[g.at(i, j, k)]; };
    std::vector<double> tmp;
    auto copyblock = [&](int di0, int di1, int dj0, int dj1, int dk0, int dk1, int si0, int sj0, int sk0) {
        int ni = di1 - di0 + 1, nj = dj1 - dj0 + 1, nk = dk1 - dk0 + 1;
        tmp.resize((size_t)ni * nj * nk);
        const long plane = (long)ni * nj;
        pfor(nk, plane, [&](int k0, int k1) {
            for (int k = k0; k < k1; ++k) { size_t c = (size_t)k * plane;
                for (int j = 0; j < nj; ++j) for (int i = 0; i < ni; ++i) tmp[c++] = A(si0 + i, sj0 + j, sk0 + k); }
        });
        pfor(nk, plane, [&](int k0, int k1) {
            for (int k = k0; k < k1; ++k) { size_t c = (size_t)k * plane;
                for (int j = 0; j < nj; ++j) for (int i = 0; i < ni; ++i) A(di0 + i, dj0 + j, dk0 + k) = tmp[c++]; }
        });
    };
    bool ex = mg.xper, ey = mg.yper;
    // neighbour ranks (mod_tiles.f90:59-106): for one rank a neighbour exists (== myrank)
    // only along periodic directions
    if (ex) copyblock(nx + 1, nx + nh, 1, ny, 1, nz, 1, 1, 1);              // east  (6)
    if (ex) copyblock(1 - nh, 0, 1, ny, 1, nz, nx - nh + 1, 1, 1);          // west  (4)
    if (ey) copyblock(1, nx, ny + 1, ny + nh, 1, nz, 1, 1, 1);              // north (8)
    if (ey) copyblock(1, nx, 1 - nh, 0, 1, nz, 1, ny - nh + 1, 1);          // south (2)
    if (ex && ey) {
        copyblock(nx + 1, nx + nh, ny + 1, ny + nh, 1, nz, 1, 1, 1);                   // (9)
        copyblock(1 - nh, 0, ny + 1, ny + nh, 1, nz, nx - nh + 1, 1, 1);               // (7)
        copyblock(nx + 1, nx + nh, 1 - nh, 0, 1, nz, 1, ny - nh + 1, 1);               // (3)
        copyblock(1 - nh, 0, 1 - nh, 0, 1, nz, nx - nh + 1, ny - nh + 1, 1);           // (1)
    }
    if (mg.zper) {
        copyblock(1 - nh, nx + nh, 1 - nh, ny + nh, 1, nh, 1 - nh, 1 - nh, nz - 2 * nh + 1);
        copyblock(1 - nh, nx + nh, 1 - nh, ny + nh, nz - nh + 1, nz, 1 - nh, 1 - nh, nh + 1);
    }
}

// basicoperators.f90:363-400
void fsmoother3d(const Mg& mg, MgLevel& g) {
    const int nx = g.nx, ny = g.ny, nz = g.nz, nh = g.nh;
    double* x = g.x.data(); double* y = g.y.data();
    const double* b = g.b.data(); const double* idiag = g.idiag.data();
    const double omega = mg.omega, cff1 = 1.0 - omega;
    const long pi = g.pi, pj = g.pj;
    pfor(nz + 2 - 2 * nh, (long)(nx + 2) * (ny + 2), [&](int k0, int k1) {
    for (int k = nh + k0; k < nh + k1; ++k)
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                long c = g.at(i, j, k);
                y[c] = (cff1 * x[c] + omega * ((x[c - 1] + x[c + 1] + x[c - pi] + x[c + pi] + x[c - pj] + x[c + pj]) - b[c]) * idiag[c]);
            }
    });
    pfor(nz - 2 * nh, (long)nx * ny, [&](int k0, int k1) {
    for (int k = nh + 1 + k0; k < nh + 1 + k1; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                long c = g.at(i, j, k);
                x[c] = (cff1 * y[c] + omega * ((y[c - 1] + y[c + 1] + y[c - pi] + y[c + pi] + y[c - pj] + y[c + pj]) - b[c]) * idiag[c]);
            }
    });
}

// basicoperators.f90:300-323
void fresidual3d(MgLevel& g) {
    const int nx = g.nx, ny = g.ny, nz = g.nz, nh = g.nh;
    const double* x = g.x.data(); const double* b = g.b.data(); const double* diag = g.diag.data();
    double* r = g.r.data(); const int* msk = g.msk.data();
    const long pi = g.pi, pj = g.pj;
    pfor(nz - 2 * nh, (long)nx * ny, [&](int k0, int k1) {
    for (int k = 1 + nh + k0; k < 1 + nh + k1; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                long c = g.at(i, j, k);
                r[c] = (double)msk[c] * (b[c] + diag[c] * x[c] - (x[c - 1] + x[c + 1] + x[c - pi] + x[c + pi] + x[c - pj] + x[c + pj]));
            }
    });
}

// basicoperators.f90:32-60
void frestrict3d(const MgLevel& f, const double* xf, MgLevel& c, double* xc, const double* coef) {
    const int nh = f.nh;
    pfor(c.nz - 2 * nh, 8L * c.nx * c.ny, [&](int q0, int q1) {
    for (int kc = 1 + nh + q0; kc < 1 + nh + q1; ++kc) {
        int k = 1 + nh + (kc - 1 - nh) * 2;
        for (int jc = 1; jc <= c.ny; ++jc) {
            int j = 1 + (jc - 1) * 2;
            for (int ic = 1; ic <= c.nx; ++ic) {
                int i = 1 + (ic - 1) * 2;
                auto X = [&](int a, int bb, int cc) { return xf[f.at(a, bb, cc)]; };
                long o = c.at(ic, jc, kc);
                xc[o] = coef[o] * (X(i, j, k) + X(i + 1, j, k) + X(i, j + 1, k) + X(i + 1, j + 1, k)
                                 + X(i, j, k + 1) + X(i + 1, j, k + 1) + X(i, j + 1, k + 1) + X(i + 1, j + 1, k + 1));
            }
        }
    }
    });
}

// basicoperators.f90:173-231
void fprolong3d(MgLevel& f, double* xf, const double* coef, const MgLevel& c, const double* xcp) {
    const int nh = f.nh;
    auto XC = [&](int a, int bb, int cc) { return xcp[c.at(a, bb, cc)]; };
    const int npairs = (f.nz - 2 * nh + 1) / 2;   // k = 1 + nh + 2q, q < npairs
    pfor(npairs, 2L * f.nx * f.ny, [&](int q0, int q1) {
    for (int k = 1 + nh + 2 * q0; k < 1 + nh + 2 * q1; k += 2) {
        int kc = nh + (k + 1 - nh) / 2;
        for (int j = 1; j <= f.ny - 1; j += 2) {
            int jc = (j + 1) / 2;
            for (int i = 1; i <= f.nx - 1; i += 2) {
                int ic = (i + 1) / 2;
                double a, b, cc;
                long o0, o1;
                a = 9 * XC(ic, jc, kc - 1) + 3 * XC(ic - 1, jc, kc - 1) + 3 * XC(ic, jc - 1, kc - 1) + XC(ic - 1, jc - 1, kc - 1);
                b = 9 * XC(ic, jc, kc) + 3 * XC(ic - 1, jc, kc) + 3 * XC(ic, jc - 1, kc) + XC(ic - 1, jc - 1, kc);
                cc = 9 * XC(ic, jc, kc + 1) + 3 * XC(ic - 1, jc, kc + 1) + 3 * XC(ic, jc - 1, kc + 1) + XC(ic - 1, jc - 1, kc + 1);
                o0 = f.at(i, j, k); o1 = f.at(i, j, k + 1);
                xf[o0] = xf[o0] + coef[o0] * (3 * b + a);
                xf[o1] = xf[o1] + coef[o1] * (3 * b + cc);

                a = 9 * XC(ic, jc, kc - 1) + 3 * XC(ic + 1, jc, kc - 1) + 3 * XC(ic, jc - 1, kc - 1) + XC(ic + 1, jc - 1, kc - 1);
                b = 9 * XC(ic, jc, kc) + 3 * XC(ic + 1, jc, kc) + 3 * XC(ic, jc - 1, kc) + XC(ic + 1, jc - 1, kc);
                cc = 9 * XC(ic, jc, kc + 1) + 3 * XC(ic + 1, jc, kc + 1) + 3 * XC(ic, jc - 1, kc + 1) + XC(ic + 1, jc - 1, kc + 1);
                o0 = f.at(i + 1, j, k); o1 = f.at(i + 1, j, k + 1);
                xf[o0] = xf[o0] + coef[o0] * (3 * b + a);
                xf[o1] = xf[o1] + coef[o1] * (3 * b + cc);

                a = 9 * XC(ic, jc, kc - 1) + 3 * XC(ic - 1, jc, kc - 1) + 3 * XC(ic, jc + 1, kc - 1) + XC(ic - 1, jc + 1, kc - 1);
                b = 9 * XC(ic, jc, kc) + 3 * XC(ic - 1, jc, kc) + 3 * XC(ic, jc + 1, kc) + XC(ic - 1, jc + 1, kc);
                cc = 9 * XC(ic, jc, kc + 1) + 3 * XC(ic - 1, jc, kc + 1) + 3 * XC(ic, jc + 1, kc + 1) + XC(ic - 1, jc + 1, kc + 1);
                o0 = f.at(i, j + 1, k); o1 = f.at(i, j + 1, k + 1);
                xf[o0] = xf[o0] + coef[o0] * (3 * b + a);
                xf[o1] = xf[o1] + coef[o1] * (3 * b + cc);

                a = 9 * XC(ic, jc, kc - 1) + 3 * XC(ic + 1, jc, kc - 1) + 3 * XC(ic, jc + 1, kc - 1) + XC(ic + 1, jc + 1, kc - 1);
                b = 9 * XC(ic, jc, kc) + 3 * XC(ic + 1, jc, kc) + 3 * XC(ic, jc + 1, kc) + XC(ic + 1, jc + 1, kc);
                cc = 9 * XC(ic, jc, kc + 1) + 3 * XC(ic + 1, jc, kc + 1) + 3 * XC(ic, jc + 1, kc + 1) + XC(ic + 1, jc + 1, kc + 1);
                o0 = f.at(i + 1, j + 1, k); o1 = f.at(i + 1, j + 1, k + 1);
                xf[o0] = xf[o0] + coef[o0] * (3 * b + a);
                xf[o1] = xf[o1] + coef[o1] * (3 * b + cc);
            }
        }
    }
    });
}

// basicoperators.f90:422-440
double fnorm3d(const MgLevel& g, const double* x) {
    double sum = 0.0;
    for (int k = 1 + g.nh; k <= g.nz - g.nh; ++k)
        for (int j = 1; j <= g.ny; ++j)
            for (int i = 1; i <= g.nx; ++i) {
                long c = g.at(i, j, k);
                sum = sum + (double)g.msk[c] * (x[c] * x[c]);
            }
    return sum;
}

// operators.f90:127-149, :151-170, :172-213, :215-244
void mg_residual(Mg& mg, int lev) { MgLevel& g = mg.L[lev]; fresidual3d(g); mg_fill(mg, g, g.r.data()); }
void mg_smooth(Mg& mg, int lev) { MgLevel& g = mg.L[lev]; fsmoother3d(mg, g); mg_fill(mg, g, g.x.data()); }
void mg_restrict(Mg& mg, int lev, bool from_r) {
    MgLevel& f = mg.L[lev]; MgLevel& c = mg.L[lev + 1];
    frestrict3d(f, from_r ? f.r.data() : f.b.data(), c, c.b.data(), c.Rcoef.data());
    std::fill(c.x.begin(), c.x.end(), 0.0);
    mg_fill(mg, c, c.b.data());
}
void mg_prolong(Mg& mg, int lev) {
    MgLevel& f = mg.L[lev]; MgLevel& c = mg.L[lev + 1];
    fprolong3d(f, f.x.data(), f.Pcoef.data(), c, c.x.data());
    mg_fill(mg, f, f.x.data());
}

// operators.f90:314-365 (apply_default_msk, compute_msk), :367-421 (Rcoef),
// :423-452 (Pcoef), :454-484 (diag), :461-505 (setup_operators)
void mg_setup_operators(Mg& mg) {
    const int L = mg.nlevels;
    for (int lev = 0; lev < L - 1; ++lev) {   // compute_msk
        MgLevel& f = mg.L[lev]; MgLevel& c = mg.L[lev + 1];
        std::fill(c.msk.begin(), c.msk.end(), 1);
        std::fill(c.Rcoef.begin(), c.Rcoef.end(), 1.0);
        for (long q = 0; q < f.size(); ++q) f.b[q] = (double)f.msk[q];
        mg_restrict(mg, lev, false);
        for (long q = 0; q < c.size(); ++q) c.msk[q] = (c.b[q] > 0.0) ? 1 : 0;
        // apply_default_msk: zero the x/y ghost sides that have no neighbour
        std::fill(c.y.begin(), c.y.end(), 1.0);
        for (int k = 1; k <= c.nz; ++k)
            for (int j = 1 - c.nh; j <= c.ny + c.nh; ++j)
                for (int i = 1 - c.nh; i <= c.nx + c.nh; ++i) {
                    bool zero = false;
                    if (!mg.xper && (i <= 0 || i >= c.nx + 1)) zero = true;
                    if (!mg.yper && (j <= 0 || j >= c.ny + 1)) zero = true;
                    if (zero) c.y[c.at(i, j, k)] = 0.0;
                }
        for (long q = 0; q < c.size(); ++q) c.msk[q] = (int)((double)c.msk[q] * c.y[q]);
        std::fill(c.y.begin(), c.y.end(), 0.0);
    }
    for (int lev = 0; lev < L - 1; ++lev) {
        MgLevel& f = mg.L[lev]; MgLevel& c = mg.L[lev + 1];
        // compute_Rcoef
        for (long q = 0; q < c.size(); ++q) c.Rcoef[q] = (double)c.msk[q];
        std::fill(f.b.begin(), f.b.end(), 1.0);
        mg_restrict(mg, lev, false);
        std::fill(c.Rcoef.begin(), c.Rcoef.end(), 0.0);
        for (long q = 0; q < c.size(); ++q) if (c.b[q] > 0.0) c.y[q] = 4.0 / c.b[q];
        for (long q = 0; q < c.size(); ++q) c.y[q] = (double)c.msk[q] * c.y[q];
        c.Rcoef = c.y;
        // compute_Pcoef
        std::fill(f.x.begin(), f.x.end(), 0.0);
        for (long q = 0; q < c.size(); ++q) c.x[q] = (double)c.msk[q];
        for (long q = 0; q < f.size(); ++q) f.Pcoef[q] = (double)f.msk[q];
        mg_prolong(mg, lev);
        std::fill(f.Pcoef.begin(), f.Pcoef.end(), 0.0);
        for (long q = 0; q < f.size(); ++q) if (f.x[q] > 0.0) f.Pcoef[q] = 1.0 / f.x[q];
        for (long q = 0; q < f.size(); ++q) f.Pcoef[q] = (double)f.msk[q] * f.Pcoef[q];
    }
    for (int lev = 0; lev < L; ++lev) {   // compute_diag
        MgLevel& g = mg.L[lev];
        for (long q = 0; q < g.size(); ++q) g.x[q] = (double)g.msk[q];
        std::fill(g.b.begin(), g.b.end(), 0.0);
        std::fill(g.diag.begin(), g.diag.end(), 0.0);
        mg_residual(mg, lev);
        for (long q = 0; q < g.size(); ++q) g.diag[q] = -g.r[q];
        std::fill(g.idiag.begin(), g.idiag.end(), 0.0);
        for (long q = 0; q < g.size(); ++q) if (g.diag[q] > 0.0) g.idiag[q] = 1.0 / g.diag[q];
        std::fill(g.x.begin(), g.x.end(), 0.0);
    }
}

// mg_setup.f90:225-307 (create_hierarchy), one rank: no glue. The reference loop ends
// only when x == 2 or y == 2; extents that never reach 2 (3*2^n) do not terminate there.
// Here coarsening also stops before an odd extent or an extent below 2 would be made.
int mg_count_levels(int nx, int ny, int stop_rule_ext) {
    int x = nx, y = ny, n = 1;
    while (true) {
        if (x == 2 || y == 2) break;
        if (stop_rule_ext && ((x % 2) || (y % 2) || x < 4 || y < 4)) break;
        x /= 2; y /= 2; ++n;
        if (n > 50) break;
    }
    return n;
}

Mg* mg_create(int nx, int ny, int nz, int topology) {
    Mg* mg = new Mg();
    mg->topology = topology;
    mg->xper = (topology == XPERIO || topology == XYPERIO || topology == XYZPERIO);
    mg->yper = (topology == YPERIO || topology == XYPERIO || topology == XYZPERIO);
    mg->zper = (topology == ZPERIO || topology == XYZPERIO);
    const int nh = mg->nh;
    int nl = mg_count_levels(nx, ny, 1);
    mg->nlevels = nl;
    mg->L.resize(nl);
    int x = nx, y = ny, z = nz + 2 * nh;
    for (int l = 0; l < nl; ++l) {
        if (l > 0) { x /= 2; y /= 2; z = z / 2 + nh; }
        MgLevel& g = mg->L[l];
        g.nx = x; g.ny = y; g.nz = z; g.nh = nh;
        g.pi = x + 2 * nh; g.pj = (long)(x + 2 * nh) * (y + 2 * nh);
        long s = g.size();
        g.x.assign(s, 0.0); g.b.assign(s, 0.0); g.r.assign(s, 0.0); g.y.assign(s, 0.0);
        g.diag.assign(s, 0.0); g.idiag.assign(s, 0.0); g.Rcoef.assign(s, 0.0); g.Pcoef.assign(s, 0.0);
        g.msk.assign(s, 0);
    }
    // set_default_msk (mg_setup.f90:180-211), is3d
    for (int l = 0; l < nl; ++l) {
        MgLevel& g = mg->L[l];
        for (int k = 1; k <= g.nz; ++k)
            for (int j = 1; j <= g.ny; ++j)
                for (int i = 1; i <= g.nx; ++i)
                    if (mg->zper || (k >= 1 + nh && k <= g.nz - nh)) g.msk[g.at(i, j, k)] = 1;
    }
    // setup_fine_msk (mg_setup.f90:213-223)
    {
        MgLevel& g = mg->L[0];
        for (long q = 0; q < g.size(); ++q) g.y[q] = (double)g.msk[q];
        mg_fill(*mg, g, g.y.data());
        for (long q = 0; q < g.size(); ++q) g.msk[q] = (int)g.y[q];
    }
    mg_setup_operators(*mg);
    return mg;
}

// solvers.f90:35-55
void mg_vcycle(Mg& mg) {
    int lev1 = mg.nlevels - 1;   // 0-based index of the coarsest level
    for (int lev = 0; lev < lev1; ++lev) {
        mg_smooth(mg, lev);
        mg_residual(mg, lev);
        mg_restrict(mg, lev, true);
    }
    mg_smooth(mg, lev1);
    for (int lev = lev1 - 1; lev >= 0; --lev) {
        mg_prolong(mg, lev);
        mg_smooth(mg, lev);
    }
}

// operators.f90:81-96
double mg_normresidual(Mg& mg, double normb) {
    if (normb > 0.0) {
        mg_residual(mg, 0);
        return fnorm3d(mg.L[0], mg.L[0].r.data()) / normb;
    }
    return 0.0;
}

// solvers.f90:8-33
void mg_solve(Mg& mg) {
    int nite = 0;
    double normb = fnorm3d(mg.L[0], mg.L[0].b.data());
    double res = mg_normresidual(mg, normb);
    while (true) {
        if (res < mg.tol) break;
        mg_vcycle(mg);
        nite = nite + 1;
        if (nite >= mg.maxite) break;
        res = mg_normresidual(mg, normb);
    }
    mg.nite = nite;
    mg.res = res;
}

// ================================================================ model
// Restatement of core/model_les.py, core/model_les_euler.py, core/timescheme.py,
// core/projection.py, core/mgfordriver.py, core/mpi/halo.py for one rank.
enum Fld { B = 0, P, KE, DIV, UX, UY, UZ, CX, CY, CZ, WX, WY, WZ, WORK, T0 };  // CX.. = contravariant U

struct Model {
    int n[3];             // interior nz, ny, nx
    int N[3];             // array extents (z, y, x)
    int per[3];           // periodic flags (z, y, x)
    int nh = 3;
    int ntr = 0;
    int model = 0;        // 0 LES, 1 Euler3d, 2 linear, 3 advection (core/model_advection.py)
    int scheme = 2;       // 0 EF, 1 LFAM3, 2 RK3_SSP
    double dx, dy, dz, idx2, idy2, idz2;
    double fparam = 0.0;  // covariant Coriolis (coriolis * dx * dy), 0 if not rotating
    double visc = 0.0; int add_visc = 0;
    // tracer diffusion (core/tracer.py:74-76), applied only when bit q of trdiff_mask is
    // set (q = 0 for b): the reference's rhs never passes `last` to rhstrac
    double kappa[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}; int trdiff_mask = 0;
    int tr_order = 0;     // 0 WENO (the reference); 1..5 the linear branch of order orderA
    int vf_order = 0;     // vortex force: 0 WENO (the reference); 1..5 the linear branch (orderVF)
    bool lfam3_first = true;
    long vol;
    std::vector<std::vector<double>> f;    // state fields (14 + ntr)
    // prognostic registers: [reg][prognostic index] ; prognostic = b, u_i, u_j, u_k, t0..
    std::vector<std::vector<std::vector<double>>> reg;   // ds0, ds1, ds2 (RK3) / dstate, stateb, staten
    Mg* mg = nullptr;
    std::vector<double> mgx, mgb;   // level-1 numpy buffers of MG.preallocate_for_nyles
    void (*forcing)(void* user, int reg, double t, void* stream) = nullptr;   // forcing.add hook
    void* forcing_user = nullptr;
    int nprog() const { return 4 + ntr; }
};

int prog_field(int q) { return q == 0 ? B : (q <= 3 ? UX + (q - 1) : T0 + (q - 4)); }

// core/mpi/halo.py:140-178 for one rank: periodic self-copy through all 26 (closed:
// fewer) directions; the send slices read only interior cells, so one copy pass over
// each halo region reproduces it.
void model_fill(const Model& M, double* a) {
    const int* N = M.N; const int nh = M.nh;
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { lo[d] = M.per[d] ? nh : 0; hi[d] = M.per[d] ? N[d] - nh : N[d]; }
    auto src = [&](int d, int c) {   // position in the interior that halo cell c mirrors
        if (!M.per[d]) return c;
        int n = M.n[d];
        if (c < nh) return c + n;
        if (c >= nh + n) return c - n;
        return c;
    };
    // halo cells only are written, interior cells only are read
    pfor(N[0], (long)N[1] * N[2], [&](int k0, int k1) {
    for (int k = k0; k < k1; ++k)
        for (int j = 0; j < N[1]; ++j)
            for (int i = 0; i < N[2]; ++i) {
                bool inside = (k >= lo[0] && k < hi[0]) && (j >= lo[1] && j < hi[1]) && (i >= lo[2] && i < hi[2]);
                if (inside) continue;
                long dst = ((long)k * N[1] + j) * N[2] + i;
                long s = ((long)src(0, k) * N[1] + src(1, j)) * N[2] + src(2, i);
                a[dst] = a[s];
            }
    });
}

V3 fv(Model& M, int fld, char d) { return view(M.f[fld].data(), M.N, d); }
V3 ffv(Model& M, int fld, char d) { return flipview(M.f[fld].data(), M.N, d); }
V3 rv(Model& M, std::vector<std::vector<double>>& r, int fld, char d) {
    int q = (fld == B) ? 0 : (fld >= T0 ? 4 + (fld - T0) : 1 + (fld - UX));
    return view(r[q].data(), M.N, d);
}
V3 rfv(Model& M, std::vector<std::vector<double>>& r, int fld, char d) {
    int q = (fld == B) ? 0 : (fld >= T0 ? 4 + (fld - T0) : 1 + (fld - UX));
    return flipview(r[q].data(), M.N, d);
}
int dirn(char d) { return d == 'i' ? 0 : (d == 'j' ? 1 : 2); }

// core/vortex_force.py:69-81
void model_vortex_force(Model& M, std::vector<std::vector<double>>& ds) {
    const char* trip[3] = {"ikj", "jik", "kji"};
    for (int t = 0; t < 3; ++t) {
        char k = trip[t][0], j = trip[t][1], i = trip[t][2];
        V3 u_i = rfv(M, ds, UX + dirn(i), j);
        V3 u_k = rfv(M, ds, UX + dirn(k), j);
        V3 U_i = ffv(M, CX + dirn(i), j);
        V3 U_k = ffv(M, CX + dirn(k), j);
        V3 w_j = ffv(M, WX + dirn(j), j);
        if (M.vf_order > 0) {
            vortex_force_direc_linear(U_k, w_j, u_i, M.vf_order);
            vortex_force_flip_linear(U_i, w_j, u_k, M.vf_order);
        } else {
            vortex_force_direc(U_k, w_j, u_i);
            vortex_force_flip(U_i, w_j, u_k);
        }
    }
}

// core/tracer.py:44-78; `last` with a tracer's bit in trdiff_mask adds its diffusion
// after each direction's advection (core/tracer.py:74-76)
void model_rhstrac(Model& M, std::vector<std::vector<double>>& ds, bool last) {
    if (M.model == 1) return;   // Euler3d: tracer step commented out (model_les_euler.py:131)
    for (int tr = 0; tr <= M.ntr; ++tr) {
        int fld = (tr == 0) ? B : T0 + tr - 1;
        for (char d : {'i', 'j', 'k'}) {
            V3 vel = fv(M, CX + dirn(d), d);
            V3 field = fv(M, fld, d);
            V3 dfield = rv(M, ds, fld, d);
            if (d == 'i') { double* p = ds[fld == B ? 0 : 4 + (fld - T0)].data(); std::fill(p, p + M.vol, 0.0); }
            if (M.tr_order > 0) upwind_linear(field, vel, dfield, M.tr_order);
            else upwind(field, vel, dfield);
            if (last && ((M.trdiff_mask >> tr) & 1)) {
                double ids2 = d == 'i' ? M.idx2 : (d == 'j' ? M.idy2 : M.idz2);
                add_laplacian(field, dfield, M.kappa[tr] * ids2);
            }
        }
    }
}

// core/bernoulli.py:14-32
void model_bernoulli(Model& M, std::vector<std::vector<double>>& ds) {
    for (char d : {'i', 'j', 'k'}) {
        V3 du = rv(M, ds, UX + dirn(d), d);
        V3 ke = fv(M, KE, d);
        if (d != 'k' || M.model == 1) gradke(ke, du);
        else gradkeandb(ke, fv(M, B, d), du, M.dz);
    }
}

// core/viscosity.py:3-9
void model_viscosity(Model& M, std::vector<std::vector<double>>& ds) {
    for (char direc : {'i', 'j', 'k'}) {
        double ids2 = direc == 'i' ? M.idx2 : (direc == 'j' ? M.idy2 : M.idz2);
        double coef = M.visc * ids2;
        for (char comp : {'i', 'j', 'k'})
            add_laplacian(fv(M, UX + dirn(comp), direc), rv(M, ds, UX + dirn(comp), direc), coef);
    }
}

// core/model_les.py:130-144, :167-175
void model_rhs(Model& M, std::vector<std::vector<double>>& ds, bool last) {
    if (M.model == 3) {   // Advection.rhs, core/model_advection.py:59-61: b only, no reset_state
        model_rhstrac(M, ds, last);
        return;
    }
    for (auto& a : ds) std::fill(a.begin(), a.end(), 0.0);
    model_rhstrac(M, ds, last);
    if (M.model != 2) model_vortex_force(M, ds);
    model_bernoulli(M, ds);
    if (last && M.add_visc) model_viscosity(M, ds);
}

// core/cov_to_contra.py:4-20
void model_U_from_u(Model& M) {
    const double c[3] = {M.idx2, M.idy2, M.idz2};
    for (int d = 0; d < 3; ++d) {
        const double* u = M.f[UX + d].data(); double* U = M.f[CX + d].data();
        const double cd = c[d];
        pfor_elems(M.vol, [&](long q) { U[q] = u[q] * cd; });
    }
}

// core/projection.py:16-29
void model_compute_div(Model& M) {
    int count = 0;
    for (char d : {'i', 'j', 'k'}) { divop(fv(M, DIV, d), fv(M, CX + dirn(d), d), count); ++count; }
}

// core/projection.py:39-87 + core/mgfordriver.py:36-78
void model_compute_p(Model& M) {
    model_compute_div(M);
    double* div = M.f[DIV].data(); double* p = M.f[P].data();
    model_fill(M, div);   // solve_directly: self.halo.fill(div)
    const int nh = M.nh;
    const MgLevel& g = M.mg->L[0];
    // b[idx] = div with idx trimming nh in closed directions; MG numpy array is
    // (nz+2nh, ny+2nh, nx+2nh) and matches the Fortran level-1 layout
    int off[3]; for (int d = 0; d < 3; ++d) off[d] = M.per[d] ? 0 : nh;
    for (int k = 0; k < M.N[0]; ++k)
        for (int j = 0; j < M.N[1]; ++j)
            for (int i = 0; i < M.N[2]; ++i) {
                long mgq = ((long)(k + off[0]) * (g.ny + 2 * nh) + (j + off[1])) * (g.nx + 2 * nh) + (i + off[2]);
                M.mgb[mgq] = div[((long)k * M.N[1] + j) * M.N[2] + i];
            }
    MgLevel& G = M.mg->L[0];
    G.b = M.mgb;                  // set_pyarray(b)
    mg_solve(*M.mg);
    M.mgx = G.x;                  // get_pyarray(x)
    double dx2 = M.dx * M.dx;
    for (int k = 0; k < M.N[0]; ++k)
        for (int j = 0; j < M.N[1]; ++j)
            for (int i = 0; i < M.N[2]; ++i) {
                long mgq = ((long)(k + off[0]) * (g.ny + 2 * nh) + (j + off[1])) * (g.nx + 2 * nh) + (i + off[2]);
                p[((long)k * M.N[1] + j) * M.N[2] + i] = M.mgx[mgq] * dx2;
            }
    for (char d : {'i', 'j', 'k'}) gradke(fv(M, P, d), fv(M, UX + dirn(d), d));
}

// core/vorticity.py:7-40
void model_vorticity(Model& M) {
    const char perm[3][2] = {{'k', 'j'}, {'i', 'k'}, {'j', 'i'}};   // dirk -> (dirj, diri)
    const char dk[3] = {'i', 'j', 'k'};
    for (int t = 0; t < 3; ++t) {
        char dirk = dk[t], dirj = perm[t][0], diri = perm[t][1];
        V3 ui = ffv(M, UX + dirn(diri), dirk);
        V3 uj = ffv(M, UX + dirn(dirj), dirk);
        V3 wk = ffv(M, WX + dirn(dirk), dirk);
        vorticity_k(ui, uj, wk);
        if (M.fparam > 0.0 && dirk == 'k') {
            for (int k = 0; k < wk.n0; ++k)
                for (int j = 0; j < wk.n1 - 1; ++j)
                    for (int i = 0; i < wk.n2 - 1; ++i) wk(k, j, i) = wk(k, j, i) + M.fparam;
        }
    }
}

// core/kinenergy.py:7-24
void model_kinenergy(Model& M) {
    const double ids2[3] = {M.idx2, M.idy2, M.idz2};
    for (char d : {'i', 'j', 'k'}) {
        V3 u = fv(M, UX + dirn(d), d);
        if (d == 'i') std::fill(M.f[KE].begin(), M.f[KE].end(), 0.0);
        kin(u, fv(M, KE, d), ids2[dirn(d)]);
    }
}

// core/model_les.py:98-127 ; core/model_les_euler.py:96-125
void model_diagnose(Model& M) {
    if (M.model == 3) {   // Advection.diagnose_var, core/model_advection.py:33-35
        model_fill(M, M.f[B].data());
        return;
    }
    if (M.model != 1) {
        model_fill(M, M.f[B].data());
        for (int d = 0; d < 3; ++d) model_fill(M, M.f[UX + d].data());
    }
    model_U_from_u(M);
    model_compute_p(M);
    for (int d = 0; d < 3; ++d) model_fill(M, M.f[UX + d].data());
    model_U_from_u(M);
    if (M.model != 2) {
        model_vorticity(M);
        model_kinenergy(M);
        for (int d = 0; d < 3; ++d) model_fill(M, M.f[WX + d].data());
        model_fill(M, M.f[KE].data());
    }
}

// Advection.make_u_divergentfree, core/model_advection.py:38-53, with the projection of
// LES.diagnose_var (the reference method calls compute_p without its `ngbs` argument and
// builds the superseded Python multigrid, so it cannot run as written)
void model_project(Model& M) {
    for (int d = 0; d < 3; ++d) model_fill(M, M.f[UX + d].data());
    model_U_from_u(M);
    model_compute_p(M);
    for (int d = 0; d < 3; ++d) model_fill(M, M.f[UX + d].data());
    model_U_from_u(M);
    model_compute_div(M);
    model_fill(M, M.f[DIV].data());
}

// right-hand side into register set `reg` at stage time t, then the user forcing
// (core/model_les.py:143-144)
void model_rhs_at(Model& M, int reg, bool last, double t) {
    model_rhs(M, M.reg[reg], last);
    if (M.forcing) M.forcing(M.forcing_user, reg, t, nullptr);
}

// core/timescheme.py:113-221
void model_forward(Model& M, double t, double dt) {
    const int np = M.nprog();
    auto S = [&](int q) { return M.f[prog_field(q)].data(); };
    if (M.scheme == 2) {   // RK3_SSP
        auto& ds0 = M.reg[0]; auto& ds1 = M.reg[1]; auto& ds2 = M.reg[2];
        model_rhs_at(M, 0, false, t);
        for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds0[q].data();
            pfor_elems(M.vol, [&](long c) { s[c] = s[c] + dt * a[c]; }); }
        model_diagnose(M);
        model_rhs_at(M, 1, false, t + dt);
        const double c2 = dt / 4.0;
        for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds0[q].data(); const double* b = ds1[q].data();
            pfor_elems(M.vol, [&](long c) { s[c] = s[c] + c2 * (b[c] - 3.0 * a[c]); }); }
        model_diagnose(M);
        model_rhs_at(M, 2, true, t + dt * 0.5);
        const double c3 = dt / 12.0;
        for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds0[q].data(); const double* b = ds1[q].data(); const double* e = ds2[q].data();
            pfor_elems(M.vol, [&](long c) { s[c] = s[c] + c3 * (8.0 * e[c] - a[c] - b[c]); }); }
        model_diagnose(M);
    } else if (M.scheme == 0) {   // EF
        auto& ds = M.reg[0];
        model_rhs_at(M, 0, true, t);
        for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds[q].data();
            for (long c = 0; c < M.vol; ++c) s[c] = s[c] + dt * a[c]; }
        model_diagnose(M);
    } else {   // LFAM3
        auto& ds = M.reg[0]; auto& sb = M.reg[1]; auto& sn = M.reg[2];
        model_rhs_at(M, 0, false, t);
        if (M.lfam3_first) {
            for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds[q].data();
                for (long c = 0; c < M.vol; ++c) { sn[q][c] = s[c]; sb[q][c] = s[c]; s[c] = s[c] + dt * a[c]; } }
            M.lfam3_first = false;
            model_diagnose(M);
        } else {
            const double two_dt = 2.0 * dt, c12 = 1.0 / 12.0;
            for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds[q].data();
                for (long c = 0; c < M.vol; ++c) {
                    sn[q][c] = s[c];
                    s[c] = sb[q][c] + two_dt * a[c];
                    s[c] = c12 * (5.0 * s[c] + 8.0 * sn[q][c] - sb[q][c]);
                    sb[q][c] = sn[q][c];
                } }
            model_diagnose(M);
            model_rhs_at(M, 0, true, t + dt * 0.5);
            for (int q = 0; q < np; ++q) { double* s = S(q); const double* a = ds[q].data();
                for (long c = 0; c < M.vol; ++c) s[c] = sn[q][c] + dt * a[c]; }
            model_diagnose(M);
        }
    }
}

}  // namespace

// ================================================================ C entry points
extern "C" {

// --- f2py-signature kernels on contiguous arrays (dims = numpy shape) -------------
// host threads of the parallel loops (n <= 0: all hardware threads); returns the count
int orc_set_threads(int n) {
    if (n <= 0) n = (int)std::thread::hardware_concurrency();
    g_threads.store(std::max(1, std::min(n, 256)));
    return g_threads.load();
}
int orc_get_threads(void) { return oracle_threads(); }
double orc_weno3(double a, double b, double c) { return weno3(a, b, c); }
double orc_weno5(double a, double b, double c, double d, double e) { return weno5(a, b, c, d, e); }
void orc_flux1d(const double* u, const double* q, double* flux, int n) { flux1d(u, q, flux, n); }
void orc_vortex_force_direc(double* U, double* vort, double* res, int m, int n, int l) {
    vortex_force_direc(contig(U, m, n, l), contig(vort, m, n, l), contig(res, m, n, l)); }
void orc_vortex_force_flip(double* U, double* vort, double* res, int m, int n, int l) {
    vortex_force_flip(contig(U, m, n, l), contig(vort, m, n, l), contig(res, m, n, l)); }
void orc_upwind(double* trac, double* u, double* dtrac, int l, int m, int n) {
    upwind(contig(trac, l, m, n), contig(u, l, m, n), contig(dtrac, l, m, n)); }
void orc_vorticity(double* ui, double* uj, double* wk, int l, int m, int n) {
    vorticity_k(contig(ui, l, m, n), contig(uj, l, m, n), contig(wk, l, m, n)); }
void orc_kin(double* u, double* ke, double ds2, int l, int m, int n) {
    kin(contig(u, l, m, n), contig(ke, l, m, n), ds2); }
void orc_gradke(double* ke, double* du, int l, int m, int n) { gradke(contig(ke, l, m, n), contig(du, l, m, n)); }
void orc_gradkeandb(double* ke, double* b, double* du, double dz, int l, int m, int n) {
    gradkeandb(contig(ke, l, m, n), contig(b, l, m, n), contig(du, l, m, n), dz); }
void orc_div(double* d, double* u, int iflag, int l, int m, int n) { divop(contig(d, l, m, n), contig(u, l, m, n), iflag); }
void orc_add_laplacian(double* phi, double* dphi, double coef, int l, int m, int n) {
    add_laplacian(contig(phi, l, m, n), contig(dphi, l, m, n), coef); }

// --- multigrid (mgfor ctypes interface restated) ----------------------------------
void* orc_mg_create(int nx, int ny, int nz, int topology) { return mg_create(nx, ny, nz, topology); }
void orc_mg_destroy(void* h) { delete (Mg*)h; }
int orc_mg_nlevels(void* h) { return ((Mg*)h)->nlevels; }
// pytools.f90:8-15: (nz_level, ny+2nh, nx+2nh) in numpy order
void orc_mg_shape(void* h, int lev, int* shape) {
    const MgLevel& g = ((Mg*)h)->L[lev - 1];
    shape[0] = g.nz; shape[1] = g.ny + 2 * g.nh; shape[2] = g.nx + 2 * g.nh; }
// pytools.f90:17-60 ; ivar 1=x 2=b 3=r 4=y 5=diag 6=idiag 7=msk 8=Rcoef 9=Pcoef
static std::vector<double>* mgvar(MgLevel& g, int ivar) {
    switch (ivar) { case 1: return &g.x; case 2: return &g.b; case 3: return &g.r; case 4: return &g.y;
        case 5: return &g.diag; case 6: return &g.idiag; case 8: return &g.Rcoef; case 9: return &g.Pcoef; }
    return nullptr; }
void orc_mg_get(void* h, int lev, int ivar, double* out) {
    MgLevel& g = ((Mg*)h)->L[lev - 1];
    if (ivar == 7) { for (long q = 0; q < g.size(); ++q) out[q] = g.msk[q]; return; }
    auto* v = mgvar(g, ivar); if (v) std::memcpy(out, v->data(), sizeof(double) * g.size()); }
void orc_mg_set(void* h, int lev, int ivar, const double* in) {
    MgLevel& g = ((Mg*)h)->L[lev - 1];
    if (ivar == 7) { for (long q = 0; q < g.size(); ++q) g.msk[q] = (int)in[q]; return; }
    auto* v = mgvar(g, ivar); if (v) std::memcpy(v->data(), in, sizeof(double) * g.size()); }
void orc_mg_params(void* h, double tol, int maxite, double omega) {
    Mg* m = (Mg*)h; m->tol = tol; m->maxite = maxite; m->omega = omega; }
void orc_mg_solve(void* h, int* nite, double* res) {
    Mg* m = (Mg*)h; mg_solve(*m); if (nite) *nite = m->nite; if (res) *res = m->res; }
void orc_mg_vcycle(void* h) { mg_vcycle(*(Mg*)h); }
void orc_mg_smooth(void* h, int lev) { mg_smooth(*(Mg*)h, lev - 1); }
void orc_mg_residual(void* h, int lev) { mg_residual(*(Mg*)h, lev - 1); }
void orc_mg_restrict(void* h, int lev) { mg_restrict(*(Mg*)h, lev - 1, true); }
void orc_mg_prolong(void* h, int lev) { mg_prolong(*(Mg*)h, lev - 1); }
double orc_mg_norm(void* h, int lev, int ivar) {
    MgLevel& g = ((Mg*)h)->L[lev - 1]; return fnorm3d(g, mgvar(g, ivar)->data()); }

// --- whole model -------------------------------------------------------------------
// geometry: bit 0 = x periodic, bit 1 = y periodic, bit 2 = z periodic
// model: 0 LES, 1 Euler3d, 2 linear ; scheme: 0 EF, 1 LFAM3, 2 RK3_SSP
void* orc_model_create(int nx, int ny, int nz, int nh, int per_bits, int ntr, int model, int scheme,
                       double dx, double dy, double dz, double idx2, double idy2, double idz2,
                       double fparam, double visc, int add_visc, int mg_topology) {
    Model* M = new Model();
    M->n[0] = nz; M->n[1] = ny; M->n[2] = nx; M->nh = nh;
    M->per[2] = per_bits & 1; M->per[1] = (per_bits >> 1) & 1; M->per[0] = (per_bits >> 2) & 1;
    for (int d = 0; d < 3; ++d) M->N[d] = M->n[d] + (M->per[d] ? 2 * nh : 0);
    M->ntr = ntr; M->model = model; M->scheme = scheme;
    M->dx = dx; M->dy = dy; M->dz = dz; M->idx2 = idx2; M->idy2 = idy2; M->idz2 = idz2;
    M->fparam = fparam; M->visc = visc; M->add_visc = add_visc;
    M->vol = (long)M->N[0] * M->N[1] * M->N[2];
    M->f.assign(T0 + ntr, std::vector<double>(M->vol, 0.0));
    M->reg.assign(3, std::vector<std::vector<double>>(M->nprog(), std::vector<double>(M->vol, 0.0)));
    M->mg = mg_create(nx, ny, nz, mg_topology);
    const MgLevel& g = M->mg->L[0];
    M->mgx.assign(g.size(), 0.0); M->mgb.assign(g.size(), 0.0);
    return M;
}
void orc_model_destroy(void* h) { Model* M = (Model*)h; delete M->mg; delete M; }
double* orc_model_field(void* h, int fld) { return ((Model*)h)->f[fld].data(); }
double* orc_model_reg(void* h, int r, int q) {
    Model* M = (Model*)h;
    if (r < 0 || r >= (int)M->reg.size() || q < 0 || q >= M->nprog()) return nullptr;
    return M->reg[r][q].data();
}
void orc_model_mg_params(void* h, double tol, int maxite, double omega) {
    Model* M = (Model*)h; M->mg->tol = tol; M->mg->maxite = maxite; M->mg->omega = omega; }
void orc_model_mg_stats(void* h, int* nite, double* res) { Model* M = (Model*)h; *nite = M->mg->nite; *res = M->mg->res; }
void* orc_model_mg(void* h) { return ((Model*)h)->mg; }
void orc_model_diagnose(void* h) { model_diagnose(*(Model*)h); }
void orc_model_vortex_force(void* h, int reg) {
    Model* M = (Model*)h; for (auto& a : M->reg[reg]) std::fill(a.begin(), a.end(), 0.0); model_vortex_force(*M, M->reg[reg]); }
void orc_model_project(void* h) { model_project(*(Model*)h); }
void orc_model_set_tracer_order(void* h, int order) { ((Model*)h)->tr_order = order; }
void orc_model_set_vf_order(void* h, int order) { ((Model*)h)->vf_order = order; }
// the f2py kernels with their `order` argument honoured (0 = WENO)
void orc_vortex_force_direc_order(double* U, double* vort, double* res, int order, int m, int n, int l) {
    V3 a = contig(U, m, n, l), b = contig(vort, m, n, l), c = contig(res, m, n, l);
    if (order > 0) vortex_force_direc_linear(a, b, c, order); else vortex_force_direc(a, b, c);
}
void orc_vortex_force_flip_order(double* U, double* vort, double* res, int order, int m, int n, int l) {
    V3 a = contig(U, m, n, l), b = contig(vort, m, n, l), c = contig(res, m, n, l);
    if (order > 0) vortex_force_flip_linear(a, b, c, order); else vortex_force_flip(a, b, c);
}
void orc_upwind_linear(double* trac, double* u, double* dtrac, int order, int l, int m, int n) {
    upwind_linear(contig(trac, l, m, n), contig(u, l, m, n), contig(dtrac, l, m, n), order); }
void orc_model_set_tracer_diffusion(void* h, const double* kappa, int mask) {
    Model* M = (Model*)h;
    for (int q = 0; q <= M->ntr; ++q) M->kappa[q] = kappa[q];
    M->trdiff_mask = mask;
}
void orc_model_rhs(void* h, int reg, int last) { Model* M = (Model*)h; model_rhs(*M, M->reg[reg], last != 0); }
void orc_model_forward(void* h, double t, double dt) { model_forward(*(Model*)h, t, dt); }
void orc_model_set_forcing(void* h, void (*fn)(void*, int, double, void*), void* user) {
    Model* M = (Model*)h; M->forcing = fn; M->forcing_user = user; }
void orc_model_fill(void* h, int fld) { Model* M = (Model*)h; model_fill(*M, M->f[fld].data()); }
// core/nyles.py:227-260
double orc_model_max_U2(void* h) {
    Model* M = (Model*)h; const double* U = M->f[CX].data(); const double* V = M->f[CY].data(); const double* W = M->f[CZ].data();
    double m = -1.0;
    for (long q = 0; q < M->vol; ++q) { double s = U[q] * U[q] + V[q] * V[q] + W[q] * W[q]; if (s > m || q == 0) m = s; }
    return m;
}

// core/online_diag.py:11-35 (VFwork.compute): the u components of the first register
// are zeroed (b is left as it is) and receive the vortex force; then, direction by
// direction (i, j, k), work += (U*F*0.5)(p) + (U*F*0.5)(p - e_d) wherever the index
// along d is >= 1, in numpy's association order; the result is summed over the box
// {k0, k1, j0, j1, i0, i1} of the (k, j, i) arrays, in plain loop order.
double orc_model_vfwork(void* h, const long long* box) {
    Model* M = (Model*)h;
    auto& ds = M->reg[0];
    for (int q = 1; q <= 3; ++q) std::fill(ds[q].begin(), ds[q].end(), 0.0);
    model_vortex_force(*M, ds);
    const int Nz = M->N[0], Ny = M->N[1], Nx = M->N[2];
    const long st[3] = {1, (long)Nx, (long)Nx * Ny};
    double* w = M->f[WORK].data();
    for (int k = 0; k < Nz; ++k)
        for (int j = 0; j < Ny; ++j)
            for (int i = 0; i < Nx; ++i) {
                const long q = ((long)k * Ny + j) * Nx + i;
                const int idx[3] = {i, j, k};
                double r = 0.0;
                for (int d = 0; d < 3; ++d) {
                    if (idx[d] < 1) continue;
                    const double* U = M->f[CX + d].data();
                    const double* F = ds[1 + d].data();
                    const double a = U[q] * F[q] * 0.5;
                    const double b = U[q - st[d]] * F[q - st[d]] * 0.5;
                    r = r + (a + b);
                }
                w[q] = r;
            }
    double s = 0.0;
    for (long long k = box[0]; k < box[1]; ++k)
        for (long long j = box[2]; j < box[3]; ++j)
            for (long long i = box[4]; i < box[5]; ++i) s += w[(k * Ny + j) * Nx + i];
    return s;
}

}  // extern "C"
