// The reference's "simple" step family (MainLoopSimple, ...SC, ...Walls,
// ...WallsSC, ...WallsGravity, ...WallsInletOutlet, ...WallsInletOutletSC;
// idpy/LBM/MultiPhase.py:164-1014): hand-written kernels whose arithmetic
// differs from the generated (Meta) step, restated here in FP64.
//
//   inlet   walls == 2: n = 2, u = (u_in, 0, ..), second-order equilibrium
//           (K_SetPopNUXInletDutyCycle, LBMKernels.py:299-357)
//   outlet  walls == 3: n, u and populations of the cell at x - 1
//           (K_SetPopNUOutletNoGradient, LBMKernels.py:423-456)
//   moments walls == 1: n = sum_q f_q, u = sum_q f_q xi_q / n (K_ComputeMomentsWalls,
//           LBMKernels.py:220-258); psi on walls != 0 (K_ComputePsiWalls,
//           MultiPhaseKernels.py:583-604)
//   collide walls == 1 (walls != 0 with gravity): Shan-Chen force from the E
//           list, then Guo forcing (u += F/(2n), stored) or the Shan-Chen
//           velocity shift (u_eq = u + F/(n omega), stored u = (u + u_post)/2);
//           gravity adds g to F_y (MultiPhaseKernels.py:132-561)
//   stream  periodic pull (K_StreamPeriodic, LBMKernels.py:117-149) and halfway
//           bounce-back out of the wall cells (K_HalfWayBounceBack, :151-185)
//
// Here the collision push-streams: a population whose target is a wall cell
// goes to the opposite population of its own cell, which is what the pull
// stream followed by the bounce-back leaves in every non-wall cell (wall cells
// are never read).  STRICT keeps every operation of the reference's C in its
// order (__dmul_rn / __dadd_rn, no contraction).  Wall flags may be null (the
// periodic loops): every cell is fluid.
//
// FP32 (the *_f32 kernels): the library's shifted storage, g_q = f_q - w_q rho0
// and dn = n - rho0, with the same formulas regrouped around the deviations
// (f_eq - w rho0 = w [dn + n (3 u.xi + 4.5 (u.xi)^2 - 1.5 u^2)]) and the rest
// population from mass conservation, as the other FP32 kernels; not a parity
// path (the FP64 kernels are).
#pragma once

#include "kernels.cuh"

namespace sclbm {

struct SimpleParams {
    Geometry<double> geo;
    double w[19];      // lattice weights (the reference's W_list)
    double we[92];     // force-stencil weights (EW_list)
    double neg_g;      // -G
    double omega;
    double g;          // gravity along y
    double u_in;       // inlet velocity along x
    double rho0;       // FP32: the storage shift (0 in FP64)
    int psi_kind;
    int gravity;       // 1: F_y += g, collide every cell with walls != 0
};

template <bool STRICT>
__device__ __forceinline__ double smul(double a, double b) {
    if constexpr (STRICT) return __dmul_rn(a, b);
    else return a * b;
}
template <bool STRICT>
__device__ __forceinline__ double sadd(double a, double b) {
    if constexpr (STRICT) return __dadd_rn(a, b);
    else return a + b;
}
template <bool STRICT>
__device__ __forceinline__ double sdiv(double a, double b) {
    if constexpr (STRICT) return __ddiv_rn(a, b);
    else return a / b;
}

__device__ __forceinline__ int flag_of(const unsigned char *walls, int64_t g) { return walls ? walls[g] : 1; }

// inlet (walls == 2): equilibrium at n = 2, u = (u_in, 0, ..)
template <class L, bool STRICT>
__global__ void __launch_bounds__(256) k_simple_inlet(double *__restrict__ pop, double *__restrict__ dn,
                                                     double *__restrict__ u, const unsigned char *__restrict__ walls,
                                                     const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        if (flag_of(walls, g) != 2) continue;
        const double ln = 2.0;
        dn[g] = ln;
        const double us = p.u_in;
        const double u_dot_u = smul<STRICT>(us, us);
        double lu[D];
        lu[0] = us;
        u[g] = us;
#pragma unroll
        for (int d = 1; d < D; d++) lu[d] = u[(int64_t)d * V + g] = 0.0;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            double ux = 0.0;
#pragma unroll
            for (int d = 0; d < D; d++) ux = sadd<STRICT>(ux, smul<STRICT>(lu[d], (double)L::xi(q, d)));
            double leq = 1.0;
            leq = sadd<STRICT>(leq, smul<STRICT>(ux, 3.0));
            leq = sadd<STRICT>(leq, smul<STRICT>(smul<STRICT>(smul<STRICT>(0.5, ux), ux), 9.0));
            leq = sadd<STRICT>(leq, -smul<STRICT>(smul<STRICT>(0.5, u_dot_u), 3.0));
            leq = smul<STRICT>(smul<STRICT>(leq, ln), p.w[q]);
            pop[(int64_t)q * V + g] = leq;
        }
    }
}

// outlet (walls == 3): copy of the cell at x - 1
template <class L, class Real>
__global__ void __launch_bounds__(256) k_simple_outlet(Real *__restrict__ pop, Real *__restrict__ dn,
                                                      Real *__restrict__ u, const unsigned char *__restrict__ walls,
                                                      const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        if (flag_of(walls, g) != 3) continue;
        const int64_t src = g - 1;  // x - 1 (the outlet column is never x = 0)
        dn[g] = dn[src];
#pragma unroll
        for (int d = 0; d < D; d++) u[(int64_t)d * V + g] = u[(int64_t)d * V + src];
#pragma unroll
        for (int q = 0; q < Q; q++) pop[(int64_t)q * V + g] = pop[(int64_t)q * V + src];
    }
}

// moments on fluid cells, psi on every non-wall cell
template <class L, bool STRICT>
__global__ void __launch_bounds__(256) k_simple_moments(const double *__restrict__ pop, double *__restrict__ dn,
                                                       double *__restrict__ u, double *__restrict__ psi,
                                                       const unsigned char *__restrict__ walls, const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const int fl = flag_of(walls, g);
        if (fl == 0) continue;
        if (fl == 1) {
            double ln = 0.0, lu[D];
#pragma unroll
            for (int d = 0; d < D; d++) lu[d] = 0.0;
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const double f = pop[(int64_t)q * V + g];
                ln = sadd<STRICT>(ln, f);
#pragma unroll
                for (int d = 0; d < D; d++) lu[d] = sadd<STRICT>(lu[d], smul<STRICT>(f, (double)L::xi(q, d)));
            }
            dn[g] = ln;
#pragma unroll
            for (int d = 0; d < D; d++) u[(int64_t)d * V + g] = sdiv<STRICT>(lu[d], ln);
        }
        psi[g] = psi_of<double>(p.psi_kind, dn[g]);
    }
}

// force + collision (+ push stream with halfway bounce-back when PUSH; in place otherwise)
template <class L, class S, bool STRICT, bool SC, bool PUSH>
__global__ void __launch_bounds__(128) k_simple_collide(const double *pop, double *pop_out,
                                                       const double *__restrict__ dn, double *__restrict__ u,
                                                       const double *__restrict__ psi,
                                                       const unsigned char *__restrict__ walls, const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    const double om = p.omega;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const int fl = flag_of(walls, g);
        if (fl == 0) continue;
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
        double f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = pop[(int64_t)q * V + g];
        const bool collide = p.gravity ? true : fl == 1;
        if (collide) {
            double F[D];
#pragma unroll
            for (int d = 0; d < D; d++) F[d] = 0.0;
            const double lpsi = psi[g];
#pragma unroll
            for (int a = 0; a < S::QE; a++) {
                const int64_t nb = index_at<D>(c, S::e(a, 0), S::e(a, 1), D == 3 ? S::e(a, 2) : 0, p.geo.L);
                const double npsi = psi[nb];
#pragma unroll
                for (int d = 0; d < D; d++)
                    F[d] = sadd<STRICT>(F[d], smul<STRICT>(smul<STRICT>((double)S::e(a, d), p.we[a]), npsi));
            }
            const double sc = smul<STRICT>(p.neg_g, lpsi);
#pragma unroll
            for (int d = 0; d < D; d++) F[d] = smul<STRICT>(F[d], sc);
            if (p.gravity) F[1] = sadd<STRICT>(F[1], p.g);
            const double ln = dn[g];
            double lu[D], u0[D];
#pragma unroll
            for (int d = 0; d < D; d++) u0[d] = u[(int64_t)d * V + g];
            if constexpr (!SC) {
#pragma unroll
                for (int d = 0; d < D; d++) {
                    lu[d] = sadd<STRICT>(u0[d], sdiv<STRICT>(smul<STRICT>(0.5, F[d]), ln));
                    u[(int64_t)d * V + g] = lu[d];
                }
                double u_dot_u = 0.0, F_dot_u = 0.0;
#pragma unroll
                for (int d = 0; d < D; d++) {
                    u_dot_u = sadd<STRICT>(u_dot_u, smul<STRICT>(lu[d], lu[d]));
                    F_dot_u = sadd<STRICT>(F_dot_u, smul<STRICT>(F[d], lu[d]));
                }
                const double a1 = 1.0 - om, a2 = 1.0 - 0.5 * om;  // constant-folded in the reference's C
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    double ux = 0.0, Fx = 0.0;
#pragma unroll
                    for (int d = 0; d < D; d++) {
                        ux = sadd<STRICT>(ux, smul<STRICT>(lu[d], (double)L::xi(q, d)));
                        Fx = sadd<STRICT>(Fx, smul<STRICT>(F[d], (double)L::xi(q, d)));
                    }
                    double leq = sadd<STRICT>(1.0, sadd<STRICT>(smul<STRICT>(ux, 3.0),
                                                                smul<STRICT>(smul<STRICT>(smul<STRICT>(0.5, ux), ux), 9.0)));
                    leq = sadd<STRICT>(leq, smul<STRICT>(smul<STRICT>(-0.5, u_dot_u), 3.0));
                    leq = smul<STRICT>(smul<STRICT>(leq, ln), p.w[q]);
                    double guo = sadd<STRICT>(0.0, sadd<STRICT>(smul<STRICT>(Fx, 3.0),
                                                                smul<STRICT>(smul<STRICT>(Fx, ux), 9.0)));
                    guo = sadd<STRICT>(guo, smul<STRICT>(-F_dot_u, 3.0));
                    guo = smul<STRICT>(guo, p.w[q]);
                    f[q] = sadd<STRICT>(sadd<STRICT>(smul<STRICT>(f[q], a1), smul<STRICT>(leq, om)),
                                        smul<STRICT>(a2, guo));
                }
            } else {
#pragma unroll
                for (int d = 0; d < D; d++) lu[d] = sadd<STRICT>(u0[d], sdiv<STRICT>(sdiv<STRICT>(F[d], ln), om));
                double u_dot_u = 0.0, up[D];
#pragma unroll
                for (int d = 0; d < D; d++) {
                    u_dot_u = sadd<STRICT>(u_dot_u, smul<STRICT>(lu[d], lu[d]));
                    up[d] = 0.0;
                }
                const double a1 = 1.0 - om;
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    double ux = 0.0;
#pragma unroll
                    for (int d = 0; d < D; d++) ux = sadd<STRICT>(ux, smul<STRICT>(lu[d], (double)L::xi(q, d)));
                    double leq = sadd<STRICT>(1.0, sadd<STRICT>(smul<STRICT>(ux, 3.0),
                                                                smul<STRICT>(smul<STRICT>(smul<STRICT>(0.5, ux), ux), 9.0)));
                    leq = sadd<STRICT>(leq, smul<STRICT>(smul<STRICT>(-0.5, u_dot_u), 3.0));
                    leq = smul<STRICT>(smul<STRICT>(leq, ln), p.w[q]);
                    f[q] = sadd<STRICT>(smul<STRICT>(f[q], a1), smul<STRICT>(leq, om));
#pragma unroll
                    for (int d = 0; d < D; d++) up[d] = sadd<STRICT>(up[d], smul<STRICT>(f[q], (double)L::xi(q, d)));
                }
#pragma unroll
                for (int d = 0; d < D; d++)
                    u[(int64_t)d * V + g] = smul<STRICT>(0.5, sadd<STRICT>(u0[d], sdiv<STRICT>(up[d], ln)));
            }
        }
        if constexpr (PUSH) {
#pragma unroll
            for (int q = 0; q < Q; q++) {
                int64_t dst = index_at<D>(c, L::xi(q, 0), L::xi(q, 1), D == 3 ? L::xi(q, 2) : 0, p.geo.L);
                int qd = q;
                if (q != 0 && flag_of(walls, dst) == 0) {
                    dst = g;
                    qd = opposite_q<L>(q);
                }
                pop_out[(int64_t)qd * V + dst] = f[q];
            }
        } else if (collide) {
#pragma unroll
            for (int q = 0; q < Q; q++) pop_out[(int64_t)q * V + g] = f[q];
        }
    }
}

// pure push stream with halfway bounce-back (the SC inlet/outlet loop streams
// before it collides)
template <class L, class Real>
__global__ void __launch_bounds__(128) k_simple_stream(const Real *__restrict__ pop, Real *__restrict__ pop_out,
                                                      const unsigned char *__restrict__ walls, const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        if (flag_of(walls, g) == 0) continue;
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
#pragma unroll
        for (int q = 0; q < Q; q++) {
            int64_t dst = index_at<D>(c, L::xi(q, 0), L::xi(q, 1), D == 3 ? L::xi(q, 2) : 0, p.geo.L);
            int qd = q;
            if (q != 0 && flag_of(walls, dst) == 0) {
                dst = g;
                qd = opposite_q<L>(q);
            }
            pop_out[(int64_t)qd * V + dst] = pop[(int64_t)q * V + g];
        }
    }
}

// ---------------------------------------------------------------------------
// FP32-shifted kernels
// ---------------------------------------------------------------------------
template <class L>
__global__ void __launch_bounds__(256) k_simple_inlet_f32(float *__restrict__ pop, float *__restrict__ dn,
                                                         float *__restrict__ u, const unsigned char *__restrict__ walls,
                                                         const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    const float rho0 = (float)p.rho0, us = (float)p.u_in;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        if (flag_of(walls, g) != 2) continue;
        const float n = 2.0f, dnv = (float)(2.0 - p.rho0);
        dn[g] = dnv;
        u[g] = us;
#pragma unroll
        for (int d = 1; d < D; d++) u[(int64_t)d * V + g] = 0.0f;
        const float u2 = us * us;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const float ux = us * (float)L::xi(q, 0);
            pop[(int64_t)q * V + g] = (float)p.w[q] * (dnv + n * (3.0f * ux + 4.5f * ux * ux - 1.5f * u2));
        }
        (void)rho0;
    }
}

template <class L>
__global__ void __launch_bounds__(256) k_simple_moments_f32(const float *__restrict__ pop, float *__restrict__ dn,
                                                           float *__restrict__ u, float *__restrict__ psi,
                                                           const unsigned char *__restrict__ walls,
                                                           const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    const float rho0 = (float)p.rho0;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const int fl = flag_of(walls, g);
        if (fl == 0) continue;
        if (fl == 1) {
            float sdn = 0.0f, lu[D];
#pragma unroll
            for (int d = 0; d < D; d++) lu[d] = 0.0f;
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const float f = pop[(int64_t)q * V + g];
                sdn += f;
#pragma unroll
                for (int d = 0; d < D; d++)
                    if (L::xi(q, d) != 0) lu[d] += L::xi(q, d) > 0 ? f : -f;
            }
            dn[g] = sdn;
            const float n = rho0 + sdn;
#pragma unroll
            for (int d = 0; d < D; d++) u[(int64_t)d * V + g] = lu[d] / n;
        }
        psi[g] = psi_of<float>(p.psi_kind, rho0 + dn[g]);
    }
}

template <class L, class S, bool SC, bool PUSH>
__global__ void __launch_bounds__(128) k_simple_collide_f32(const float *pop, float *pop_out,
                                                           const float *__restrict__ dn, float *__restrict__ u,
                                                           const float *__restrict__ psi,
                                                           const unsigned char *__restrict__ walls,
                                                           const SimpleParams p) {
    constexpr int D = L::D, Q = L::Q;
    const int64_t V = p.geo.V;
    const float om = (float)p.omega, rho0 = (float)p.rho0, neg_g = (float)p.neg_g;
    const float a1 = (float)(1.0 - p.omega), a2 = (float)(1.0 - 0.5 * p.omega);
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const int fl = flag_of(walls, g);
        if (fl == 0) continue;
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
        float f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = pop[(int64_t)q * V + g];
        const bool collide = p.gravity ? true : fl == 1;
        if (collide) {
            float F[D];
#pragma unroll
            for (int d = 0; d < D; d++) F[d] = 0.0f;
#pragma unroll
            for (int a = 0; a < S::QE; a++) {
                const int64_t nb = index_at<D>(c, S::e(a, 0), S::e(a, 1), D == 3 ? S::e(a, 2) : 0, p.geo.L);
                const float npsi = psi[nb];
#pragma unroll
                for (int d = 0; d < D; d++)
                    if (S::e(a, d) != 0) F[d] = fmaf((float)(S::e(a, d) * p.we[a]), npsi, F[d]);
            }
            const float sc = neg_g * psi[g];
#pragma unroll
            for (int d = 0; d < D; d++) F[d] *= sc;
            if (p.gravity) F[1] += (float)p.g;
            const float dnv = dn[g], n = rho0 + dnv;
            float lu[D], u0[D];
#pragma unroll
            for (int d = 0; d < D; d++) u0[d] = u[(int64_t)d * V + g];
            float rest = dnv, up[D];
#pragma unroll
            for (int d = 0; d < D; d++) {
                lu[d] = SC ? u0[d] + F[d] / n / om : u0[d] + 0.5f * F[d] / n;
                if (!SC) u[(int64_t)d * V + g] = lu[d];
                up[d] = 0.0f;
            }
            float u2 = 0.0f, uF = 0.0f;
#pragma unroll
            for (int d = 0; d < D; d++) {
                u2 = fmaf(lu[d], lu[d], u2);
                uF = fmaf(F[d], lu[d], uF);
            }
#pragma unroll
            for (int q = 1; q < Q; q++) {
                float ux = 0.0f, Fx = 0.0f;
#pragma unroll
                for (int d = 0; d < D; d++)
                    if (L::xi(q, d) != 0) {
                        ux += L::xi(q, d) > 0 ? lu[d] : -lu[d];
                        Fx += L::xi(q, d) > 0 ? F[d] : -F[d];
                    }
                const float wq = (float)p.w[q];
                const float eqd = wq * (dnv + n * (3.0f * ux + 4.5f * ux * ux - 1.5f * u2));
                float out = fmaf(f[q], a1, om * eqd);
                if (!SC) out = fmaf(a2, wq * (3.0f * Fx + 9.0f * Fx * ux - 3.0f * uF), out);
                f[q] = out;
                rest = __fsub_rn(rest, out);
#pragma unroll
                for (int d = 0; d < D; d++)
                    if (L::xi(q, d) != 0) up[d] += L::xi(q, d) > 0 ? out : -out;
            }
            f[0] = rest;  // the collision conserves mass
            if (SC) {
#pragma unroll
                for (int d = 0; d < D; d++) u[(int64_t)d * V + g] = 0.5f * (u0[d] + up[d] / n);
            }
        }
        if constexpr (PUSH) {
#pragma unroll
            for (int q = 0; q < Q; q++) {
                int64_t dst = index_at<D>(c, L::xi(q, 0), L::xi(q, 1), D == 3 ? L::xi(q, 2) : 0, p.geo.L);
                int qd = q;
                if (q != 0 && flag_of(walls, dst) == 0) {
                    dst = g;
                    qd = opposite_q<L>(q);
                }
                pop_out[(int64_t)qd * V + dst] = f[q];
            }
        } else if (collide) {
#pragma unroll
            for (int q = 0; q < Q; q++) pop_out[(int64_t)q * V + g] = f[q];
        }
    }
}

}  // namespace sclbm
