// sm_103a kernels of the Shan-Chen step: SoA populations pop[q*V + g],
// g = x + Lx*(y + Ly*z), periodic box, push streaming (as the reference,
// idpy/LBM/Collisions.py:383-561), two passes per step:
//   pass 1  k_density_psi : n = rho0 + sum_q g_q, psi = psi(n)
//   pass 2  k_fcs         : Shan-Chen force, Guo-shifted velocity, collision
//                           (expanded-operator tables), push stream
// Real = double: plain FP64 (rho0 = 0, storage f_q).  Real = float: FP32
// storage of the deviations g_q = f_q - w_q rho0 (the shift only enters the
// density monomial, see coeffs.cpp).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>

#include "lattice.cuh"

namespace sclbm {

enum { PSI_EXP_INV = 0, PSI_ONE_MINUS_EXP = 1, PSI_IDENTITY = 2 };

template <class Real>
struct Geometry {
    int L[3];
    int64_t V;
};

template <class L, class S, class Real>
struct StepParams {
    static constexpr int D = L::D, Q = L::Q, QE = S::QE, K = Mono<L::D>::K;
    Geometry<Real> geo;
    Real rho0;      // storage shift (0 for FP64)
    Real neg_g;     // -G
    int psi_kind;
    int a_nonzero;  // BGK: 1 - omega != 0
    int factored;   // FP64 BGK (SCLBM_LIT_FACTORED): the collision factored by opposite directions
    Real sw[QE][D]; // signed force weights e_{a,d} * w_a
    Real A[Q][Q];   // population operator (BGK: diagonal used)
    Real B[Q][K];   // monomial coefficients
    // factored BGK (single-pass FP32 kernel): omega, 1.5 omega, 3 omega,
    // 4.5 omega, 9 (1 - omega/2), 3 (1 - omega/2), lattice weights
    Real omega, om15, om3, om45, fc, fd;
    Real wq[Q];
};

template <class L, class Real>
struct EqParams {
    static constexpr int D = L::D, Q = L::Q, K = Mono<L::D>::K;
    Geometry<Real> geo;
    Real rho0;
    Real B[Q][K];
};

template <class Real>
__device__ __forceinline__ Real psi_of(int kind, Real n);
template <>
__device__ __forceinline__ double psi_of<double>(int kind, double n) {
    if (kind == PSI_EXP_INV) return exp(-1. / n);
    if (kind == PSI_ONE_MINUS_EXP) return 1. - exp(-n);
    return n;
}
template <>
__device__ __forceinline__ float psi_of<float>(int kind, float n) {
    if (kind == PSI_EXP_INV) return expf(-1.f / n);
    if (kind == PSI_ONE_MINUS_EXP) return 1.f - expf(-n);
    return n;
}

__device__ __forceinline__ int wrapc(int x, int L) {
    x += (x < 0) ? L : 0;
    x -= (x >= L) ? L : 0;
    return x;
}

template <int D>
struct Cell {
    int x, y, z;
};

template <int D>
__device__ __forceinline__ bool cell_of(int64_t g, const int *Ls, Cell<D> &c) {
    if (D == 2) {
        c.x = (int)(g % Ls[0]);
        c.y = (int)(g / Ls[0]);
        c.z = 0;
    } else {
        const int64_t xy = (int64_t)Ls[0] * Ls[1];
        c.z = (int)(g / xy);
        const int r = (int)(g - (int64_t)c.z * xy);
        c.y = r / Ls[0];
        c.x = r - c.y * Ls[0];
    }
    return true;
}

template <int D>
__device__ __forceinline__ int64_t index_at(const Cell<D> &c, int dx, int dy, int dz, const int *Ls) {
    const int x = wrapc(c.x + dx, Ls[0]);
    const int y = wrapc(c.y + dy, Ls[1]);
    if (D == 2) return (int64_t)x + (int64_t)Ls[0] * y;
    const int z = wrapc(c.z + dz, Ls[2]);
    return (int64_t)x + (int64_t)Ls[0] * (y + (int64_t)Ls[1] * z);
}

// population i of the reference's summation order: its generated C names them
// pop_0 .. pop_{Q-1} and sympy prints sums sorted by name ('pop_10' < 'pop_2')
template <int Q>
SCLBM_HD constexpr int lex_q(int i) {
    if (Q <= 10) return i;
    constexpr int t19[19] = {0, 1, 10, 11, 12, 13, 14, 15, 16, 17, 18, 2, 3, 4, 5, 6, 7, 8, 9};
    return t19[i];
}

// ---------------------------------------------------------------------------
// pass 1: density (deviation) and pseudopotential
// ---------------------------------------------------------------------------
template <class L, class Real>
__global__ void __launch_bounds__(256) k_density_psi(const Real *__restrict__ pop, Real *__restrict__ dn,
                                                    Real *__restrict__ psi, Geometry<Real> geo, Real rho0,
                                                    int psi_kind) {
    const int64_t V = geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        // summed in the reference's order (plain adds are never reassociated)
        Real s = pop[(int64_t)lex_q<L::Q>(0) * V + g];
#pragma unroll
        for (int i = 1; i < L::Q; i++) s += pop[(int64_t)lex_q<L::Q>(i) * V + g];
        dn[g] = s;
        psi[g] = psi_of<Real>(psi_kind, rho0 + s);
    }
}

// Shan-Chen force at a cell from the psi field
template <class L, class S, class Real, class P>
__device__ __forceinline__ void sc_force(const Real *__restrict__ psi, const Cell<L::D> &c, int64_t g,
                                         const P &p, Real *F) {
    constexpr int D = L::D;
#pragma unroll
    for (int d = 0; d < D; d++) F[d] = Real(0);
#pragma unroll
    for (int a = 0; a < S::QE; a++) {
        const int64_t nb = index_at<D>(c, S::e(a, 0), S::e(a, 1), D == 3 ? S::e(a, 2) : 0, p.geo.L);
        const Real ps = __ldg(psi + nb);
#pragma unroll
        for (int d = 0; d < D; d++)
            if (S::e(a, d) != 0) F[d] = fma(p.sw[a][d], ps, F[d]);
    }
    const Real s = p.neg_g * __ldg(psi + g);
#pragma unroll
    for (int d = 0; d < D; d++) F[d] *= s;
}

// ---------------------------------------------------------------------------
// Reference arithmetic (FP64, SCLBM_LIT_ROUND15): every sum in the order the
// reference's generated C evaluates it (sympy prints terms sorted by name, so
// 'pop_10' precedes 'pop_2'), every product associated left to right, and no
// contraction into FMA (__dadd_rn / __dmul_rn are never fused).  With the
// same literals, the only remaining difference to the reference is the libm
// exp() of the pseudopotential.
// ---------------------------------------------------------------------------
template <class L>
__device__ __forceinline__ double strict_density(const double *f) {
    double s = f[lex_q<L::Q>(0)];
#pragma unroll
    for (int i = 1; i < L::Q; i++) s = __dadd_rn(s, f[lex_q<L::Q>(i)]);
    return s;
}

template <class L, class S, class P>
__device__ __forceinline__ void strict_force(const double *__restrict__ psi, const Cell<L::D> &c, int64_t g,
                                             const P &p, double *F) {
    constexpr int D = L::D;
#pragma unroll
    for (int d = 0; d < D; d++) F[d] = 0.0;
#pragma unroll
    for (int a = 0; a < S::QE; a++) {
        const int64_t nb = index_at<D>(c, S::e(a, 0), S::e(a, 1), D == 3 ? S::e(a, 2) : 0, p.geo.L);
        const double ps = __ldg(psi + nb);
#pragma unroll
        for (int d = 0; d < D; d++) {
            if (S::e(a, d) == 0) continue;
            const double t = __dmul_rn(fabs(p.sw[a][d]), ps);
            F[d] = S::e(a, d) > 0 ? __dadd_rn(F[d], t) : __dsub_rn(F[d], t);
        }
    }
    const double s = __dmul_rn(p.neg_g, __ldg(psi + g));
#pragma unroll
    for (int d = 0; d < D; d++) F[d] = __dmul_rn(F[d], s);
}

template <class L>
__device__ __forceinline__ void strict_velocity(const double *f, double n, const double *F, double *u) {
    constexpr int D = L::D;
#pragma unroll
    for (int d = 0; d < D; d++) {
        double j = 0.0;
        bool first = true;
#pragma unroll
        for (int i = 0; i < L::Q; i++) {
            const int q = lex_q<L::Q>(i);
            const int x = L::xi(q, d);
            if (x == 0) continue;
            if (first) j = x > 0 ? f[q] : -f[q];
            else j = x > 0 ? __dadd_rn(j, f[q]) : __dsub_rn(j, f[q]);
            first = false;
        }
        u[d] = __dadd_rn(__ddiv_rn(j, n), __ddiv_rn(__dmul_rn(0.5, F[d]), n));
    }
}

// one term of the expanded collision, reference association ((c*x1)*x2)*x3
template <int D>
__device__ __forceinline__ double strict_term(int k, double c, double n, const double *u, const double *F) {
    using M = Mono<D>;
    if (k == 0) return __dmul_rn(c, n);
    if (k < M::NUU) return __dmul_rn(__dmul_rn(c, n), u[k - M::NU]);
    if (k < M::F) {
#pragma unroll
        for (int a = 0; a < D; a++)
#pragma unroll
            for (int b = a; b < D; b++)
                if (M::nuu(a, b) == k) return __dmul_rn(__dmul_rn(__dmul_rn(c, n), u[a]), u[b]);
        return 0.0;
    }
    if (k < M::FU) return __dmul_rn(c, F[k - M::F]);
    const int a = (k - M::FU) / D, b = (k - M::FU) % D;
    return __dmul_rn(__dmul_rn(c, F[a]), u[b]);
}

// monomials in the reference's print order: d_psi_a (then d_psi_a*lu_0_b), ln_0,
// ln_0*lu_0_a (then ln_0*lu_0_a*lu_0_b, b >= a)
template <int D>
struct PrintOrder {
    int v[Mono<D>::K];
    constexpr PrintOrder() : v() {
        using M = Mono<D>;
        int pos = 0;
        for (int a = 0; a < D; a++) {
            v[pos++] = M::F + a;
            for (int b = 0; b < D; b++) v[pos++] = M::FU + a * D + b;
        }
        v[pos++] = 0;
        for (int a = 0; a < D; a++) {
            v[pos++] = M::NU + a;
            for (int b = a; b < D; b++) v[pos++] = M::nuu(a, b);
        }
    }
};
// (a table built once by the front end: a search per unrolled use would be
// folded again at every call site by the device compiler)
template <int D>
SCLBM_HD constexpr int print_order(int i) {
    constexpr PrintOrder<D> t{};
    return t.v[i];
}

// Guo-shifted velocity: u = (sum_q xi_q f_q + F/2) / n
template <class L, class Real>
__device__ __forceinline__ void velocity(const Real *f, Real n, const Real *F, Real *u) {
    constexpr int D = L::D;
    const Real inv = Real(1) / n;
#pragma unroll
    for (int d = 0; d < D; d++) {
        Real j = Real(0);
#pragma unroll
        for (int q = 0; q < L::Q; q++) {
            if (L::xi(q, d) > 0) j += f[q];
            if (L::xi(q, d) < 0) j -= f[q];
        }
        u[d] = (j + Real(0.5) * F[d]) * inv;
    }
}

template <int D, class Real>
__device__ __forceinline__ void monomials(Real dn, Real n, const Real *u, const Real *F, Real *m) {
    using M = Mono<D>;
    m[0] = dn;
#pragma unroll
    for (int a = 0; a < D; a++) m[M::NU + a] = n * u[a];
#pragma unroll
    for (int a = 0; a < D; a++)
#pragma unroll
        for (int b = a; b < D; b++) m[M::nuu(a, b)] = m[M::NU + a] * u[b];
#pragma unroll
    for (int a = 0; a < D; a++) m[M::F + a] = F[a];
#pragma unroll
    for (int a = 0; a < D; a++)
#pragma unroll
        for (int b = 0; b < D; b++) m[M::FU + a * D + b] = F[a] * u[b];
}

// ---------------------------------------------------------------------------
// pass 2: force + collision + push stream
// ---------------------------------------------------------------------------
template <class L, class S, bool MRT, class Real, bool STRICT>
__device__ __forceinline__ void collide_cell(const Real *f, Real d, Real n, const Real *u, const Real *F, int q,
                                             const StepParams<L, S, Real> &p, Real &out) {
    constexpr int D = L::D, Q = L::Q, K = Mono<D>::K;
    if constexpr (STRICT) {
        // reference order: monomial terms, then the population terms
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < K; i++) {
            const int k = print_order<D>(i);
            if (!MRT && !bgk_nonzero<L>(q, k)) continue;
            acc = __dadd_rn(acc, strict_term<D>(k, p.B[q][k], d, u, F));
        }
        if (MRT) {
#pragma unroll
            for (int i = 0; i < Q; i++) {
                const int j = lex_q<Q>(i);
                acc = __dadd_rn(acc, __dmul_rn(p.A[q][j], f[j]));
            }
        } else if (p.a_nonzero) {
            acc = __dadd_rn(acc, __dmul_rn(p.A[q][q], f[q]));
        }
        out = acc;
    } else {
        Real m[K];
        monomials<D, Real>(d, n, u, F, m);
        Real acc = Real(0);
        if (MRT) {
#pragma unroll
            for (int j = 0; j < Q; j++) acc = fma(p.A[q][j], f[j], acc);
        } else if (p.a_nonzero) {
            acc = p.A[q][q] * f[q];
        }
#pragma unroll
        for (int k = 0; k < K; k++)
            if (MRT || bgk_nonzero<L>(q, k)) acc = fma(p.B[q][k], m[k], acc);
        out = acc;
    }
}

// index of the lattice velocity opposite to xi_q (a table built once per lattice)
template <class L>
struct OppositeQ {
    int v[L::Q];
    constexpr OppositeQ() : v() {
        for (int q = 0; q < L::Q; q++) {
            v[q] = q;
            for (int k = 0; k < L::Q; k++) {
                bool same = true;
                for (int d = 0; d < L::D; d++) same = same && (L::xi(k, d) == -L::xi(q, d));
                if (same) {
                    v[q] = k;
                    break;
                }
            }
        }
    }
};
template <class L>
SCLBM_HD constexpr int opposite_q(int q) {
    constexpr OppositeQ<L> t{};
    return t.v[q];
}

// BGK + Guo in FP64 with the operator factored by opposite directions (the
// single FP32 pass uses the same form): with c2 = 1/3, eu = xi_q.u, eF = xi_q.F,
//   f*_q = (1-w) f_q + w_q [C0 + eu (a eu + b + c eF) + d eF],
//   C0 = w n - 1.5 w n u^2 - 3 (1-w/2) u.F, a = 4.5 w n, b = 3 w n,
//   c = 9 (1-w/2), d = 3 (1-w/2)
// (the 2nd-order Hermite equilibrium plus the Guo term, Collisions.py:163-185,
// Forcings.py:104-127); a direction and its opposite share the even part
// C0 + a eu^2 + c eu eF and take the odd part b eu + d eF with opposite signs.
// FP64 storage has no shift (rho0 = 0), so d = n.  Exact coefficients, FMA:
// equal to the expanded form up to rounding.
template <class L, class S>
__device__ __forceinline__ void bgk_factored(const double *f, double d, double n, const double *u,
                                             const double *F, const StepParams<L, S, double> &p, double *out) {
    constexpr int D = L::D, Q = L::Q;
    double u2 = 0.0, uF = 0.0;
#pragma unroll
    for (int c = 0; c < D; c++) {
        u2 = fma(u[c], u[c], u2);
        uF = fma(u[c], F[c], uF);
    }
    const double C0 = p.omega * d - p.om15 * n * u2 - p.fd * uF;
    const double a = p.om45 * n, b = p.om3 * n;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int qb = opposite_q<L>(q);
        if (qb < q) continue;
        double eu = 0.0, eF = 0.0;
#pragma unroll
        for (int c = 0; c < D; c++) {
            if (L::xi(q, c) > 0) { eu += u[c]; eF += F[c]; }
            if (L::xi(q, c) < 0) { eu -= u[c]; eF -= F[c]; }
        }
        const double even = C0 + eu * fma(a, eu, p.fc * eF);
        const double odd = fma(b, eu, p.fd * eF);
        const double rq = p.wq[q] * (even + odd);
        out[q] = p.a_nonzero ? fma(p.A[q][q], f[q], rq) : rq;
        if (qb != q) {
            const double rqb = p.wq[qb] * (even - odd);
            out[qb] = p.a_nonzero ? fma(p.A[qb][qb], f[qb], rqb) : rqb;
        }
    }
}

template <class L, class S, class Real, bool STRICT>
__device__ __forceinline__ void force_velocity(const Real *__restrict__ psi, const Cell<L::D> &c, int64_t g,
                                               const StepParams<L, S, Real> &p, const Real *f, Real n, Real *F,
                                               Real *u) {
    if constexpr (STRICT) {
        strict_force<L, S>(psi, c, g, p, F);
        strict_velocity<L>(f, n, F, u);
    } else {
        sc_force<L, S, Real>(psi, c, g, p, F);
        velocity<L, Real>(f, n, F, u);
    }
}

template <class L, class S, bool MRT, class Real, bool STRICT>
__global__ void __launch_bounds__(128) k_fcs(const Real *__restrict__ pop, Real *__restrict__ pop_out,
                                            const Real *__restrict__ dn, const Real *__restrict__ psi,
                                            const __grid_constant__ StepParams<L, S, Real> p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
        Real f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = __ldg(pop + (int64_t)q * V + g);
        const Real d = __ldg(dn + g);
        const Real n = p.rho0 + d;
        Real F[D], u[D];
        force_velocity<L, S, Real, STRICT>(psi, c, g, p, f, n, F, u);
        Real out[Q];
        bool done = false;
        if constexpr (!MRT && !STRICT && std::is_same<Real, double>::value) {
            if (p.factored) {
                bgk_factored<L, S>(f, d, n, u, F, p, out);
                done = true;
            }
        }
        if (!done) {
#pragma unroll
            for (int q = 0; q < Q; q++) collide_cell<L, S, MRT, Real, STRICT>(f, d, n, u, F, q, p, out[q]);
        }
        if constexpr (std::is_same<Real, float>::value) {
            // FP32 storage: rest population from mass conservation (as the single-pass kernel)
            Real rest = d;
#pragma unroll
            for (int q = 1; q < Q; q++) rest = __fsub_rn(rest, out[q]);  // never contracted
            out[0] = rest;
        }
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int64_t dst = index_at<D>(c, L::xi(q, 0), L::xi(q, 1), D == 3 ? L::xi(q, 2) : 0, p.geo.L);
            pop_out[(int64_t)q * V + dst] = out[q];
        }
    }
}

// ---------------------------------------------------------------------------
// walls (GetWalls / MainLoopWalls, idpy/LBM/MultiPhase.py:157-162,1226-1309):
// walls[g] = 1 fluid, 0 wall.  Density and psi on fluid cells only (walls keep
// the psi they were given, K_ComputeDensityPsiWallsMeta,
// MultiPhaseKernelsMeta.py:42-105); the step on fluid cells only, a population
// whose push target is a wall going to the opposite population of its own cell
// (halfway bounce-back, Collisions.py:705-860).  Wall cells carry their
// populations unchanged from buffer to buffer (the reference leaves them
// stale), so the total mass stays constant.
// ---------------------------------------------------------------------------

template <class L, class Real>
__global__ void __launch_bounds__(256) k_density_psi_walls(const Real *__restrict__ pop, Real *__restrict__ dn,
                                                          Real *__restrict__ psi,
                                                          const unsigned char *__restrict__ walls,
                                                          const Real *__restrict__ psi_w, Geometry<Real> geo,
                                                          Real rho0, int psi_kind) {
    const int64_t V = geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        if (walls[g] != 1) {
            psi[g] = psi_w[g];  // walls keep the psi they were given
            continue;
        }
        Real s = pop[(int64_t)lex_q<L::Q>(0) * V + g];
#pragma unroll
        for (int i = 1; i < L::Q; i++) s += pop[(int64_t)lex_q<L::Q>(i) * V + g];
        dn[g] = s;
        psi[g] = psi_of<Real>(psi_kind, rho0 + s);
    }
}

template <class L, class S, bool MRT, class Real, bool STRICT>
__global__ void __launch_bounds__(128) k_fcs_walls(const Real *__restrict__ pop, Real *__restrict__ pop_out,
                                                  const Real *__restrict__ dn, const Real *__restrict__ psi,
                                                  const unsigned char *__restrict__ walls,
                                                  const __grid_constant__ StepParams<L, S, Real> p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        Real f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = __ldg(pop + (int64_t)q * V + g);
        if (walls[g] != 1) {
#pragma unroll
            for (int q = 0; q < Q; q++) pop_out[(int64_t)q * V + g] = f[q];
            continue;
        }
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
        const Real d = __ldg(dn + g);
        const Real n = p.rho0 + d;
        Real F[D], u[D];
        force_velocity<L, S, Real, STRICT>(psi, c, g, p, f, n, F, u);
        Real out[Q];
        bool done = false;
        if constexpr (!MRT && !STRICT && std::is_same<Real, double>::value) {
            if (p.factored) {
                bgk_factored<L, S>(f, d, n, u, F, p, out);
                done = true;
            }
        }
        if (!done) {
#pragma unroll
            for (int q = 0; q < Q; q++) collide_cell<L, S, MRT, Real, STRICT>(f, d, n, u, F, q, p, out[q]);
        }
        if constexpr (std::is_same<Real, float>::value) {
            Real rest = d;
#pragma unroll
            for (int q = 1; q < Q; q++) rest = __fsub_rn(rest, out[q]);
            out[0] = rest;
        }
#pragma unroll
        for (int q = 0; q < Q; q++) {
            int64_t dst = index_at<D>(c, L::xi(q, 0), L::xi(q, 1), D == 3 ? L::xi(q, 2) : 0, p.geo.L);
            int qd = q;
            if (q != 0 && walls[dst] == 0) {
                dst = g;
                qd = opposite_q<L>(q);
            }
            pop_out[(int64_t)qd * V + dst] = out[q];
        }
    }
}

// ---------------------------------------------------------------------------
// moments read-back: Guo-shifted velocity (and n) after the force
// ---------------------------------------------------------------------------
template <class L, class S, class Real, bool STRICT>
__global__ void __launch_bounds__(128) k_velocity(const Real *__restrict__ pop, const Real *__restrict__ dn,
                                                 const Real *__restrict__ psi, Real *__restrict__ u_out,
                                                 const __grid_constant__ StepParams<L, S, Real> p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
        Real f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = pop[(int64_t)q * V + g];
        const Real n = p.rho0 + dn[g];
        Real F[D], u[D];
        force_velocity<L, S, Real, STRICT>(psi, c, g, p, f, n, F, u);
#pragma unroll
        for (int d = 0; d < D; d++) u_out[(int64_t)d * V + g] = u[d];
    }
}

// ---------------------------------------------------------------------------
// equilibrium initialisation from (dn, u)
// ---------------------------------------------------------------------------
template <class L, class Real, bool STRICT>
__global__ void __launch_bounds__(128) k_init_pop(Real *__restrict__ pop, const Real *__restrict__ dn,
                                                 const Real *__restrict__ u_in,
                                                 const __grid_constant__ EqParams<L, Real> p) {
    constexpr int D = L::D, Q = L::Q, K = Mono<D>::K;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const Real d = dn[g];
        const Real n = p.rho0 + d;
        Real u[D], F[D];
#pragma unroll
        for (int a = 0; a < D; a++) { u[a] = u_in[(int64_t)a * V + g]; F[a] = Real(0); }
        if constexpr (STRICT) {
            // the reference forms n*u_a and n*u_a*u_b first, then multiplies by the literal
#pragma unroll
            for (int q = 0; q < Q; q++) {
                double acc = 0.0;
#pragma unroll
                for (int i = 0; i < K; i++) {
                    const int k = print_order<D>(i);
                    if (k >= Mono<D>::F) continue;
                    double prod = d;
                    if (k >= Mono<D>::NU && k < Mono<D>::NUU) prod = __dmul_rn(d, u[k - Mono<D>::NU]);
                    if (k >= Mono<D>::NUU) {
#pragma unroll
                        for (int a = 0; a < D; a++)
#pragma unroll
                            for (int b = a; b < D; b++)
                                if (Mono<D>::nuu(a, b) == k) prod = __dmul_rn(__dmul_rn(d, u[a]), u[b]);
                    }
                    acc = __dadd_rn(acc, __dmul_rn(p.B[q][k], prod));
                }
                pop[(int64_t)q * V + g] = acc;
            }
        } else {
            Real m[K];
            monomials<D, Real>(d, n, u, F, m);
#pragma unroll
            for (int q = 0; q < Q; q++) {
                Real acc = Real(0);
#pragma unroll
                for (int k = 0; k < Mono<D>::F; k++) acc = fma(p.B[q][k], m[k], acc);
                pop[(int64_t)q * V + g] = acc;
            }
        }
    }
}

}  // namespace sclbm
