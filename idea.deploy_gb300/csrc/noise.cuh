// Fluctuating Shan-Chen step (Gross et al. 2011): the BGK + Guo push step of
// k_fcs plus, for every population, a noise population built from Gaussian
// random moments drawn from per-cell congruential generators.
//
// Reference: MainLoopGross2011SRT (idpy/LBM/MultiPhase.py:1404-1541) and its
// kernel K_ForceGross2011CollideStreamSCMPMeta
// (idpy/LBM/MultiPhaseKernelsMeta.py:1369-1557):
//   * random moments Rm_k, k = 0 .. Q-D-2, one per non-conserved W-orthogonal
//     Hermite moment (GrossShanChenMultiPhase, idpy/LBM/Fluctuations.py:40-165):
//         Rm_k = sqrt(-2 var_k log(u0)) cos(2 pi u1) + 0
//     (Box-Muller, CRNGS.py:924-1058) from two uniforms u = state / RANDMAX of
//     one generator drawn twice, or of generators 2k and 2k+1 drawn once each
//     ("independent Gaussians", MultiPhase.py:2041-2047);
//   * generators (CRNGS.py:603-735): MINSTD (Park-Miller 16807 mod 2^31-1, the
//     64-bit product form), NUMREC (x 1664525 + 1013904223 mod 2^32), MMIX
//     (x 6364136223846793005 + 1442695040888963407 mod 2^64); each cell's
//     states are read before and written back after its update (CRNGS.py:1061-1113);
//   * the noise population rpop_q = sum_k coef[q][k] Rm_k is added after the
//     collided value, term by term in the order sympy prints the sum (moment
//     names Rm_0, Rm_1, Rm_10, ... sorted as strings; Collisions.py:526-527).
//
// Generator states live in HBM stream-major, seeds[s * V + cell] (the
// reference's 'gpu' ordering, MultiPhase.py:1962-1963): a warp's loads and
// stores of one stream are contiguous.  MMIX keeps 64-bit states, MINSTD and
// NUMREC 32-bit ones.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

#include "kernels.cuh"

namespace sclbm {

enum : int { CRNG_MINSTD = 1, CRNG_NUMREC = 2, CRNG_MMIX = 3 };

// i-th moment index when the names Rm_0 .. Rm_{n-1} are sorted as strings
SCLBM_HD constexpr int digits_of(int v, int *d) {
    int n = 0;
    int t[12] = {};
    do {
        t[n++] = v % 10;
        v /= 10;
    } while (v > 0);
    for (int i = 0; i < n; i++) d[i] = t[n - 1 - i];
    return n;
}
SCLBM_HD constexpr bool name_less(int a, int b) {
    int da[12] = {}, db[12] = {};
    const int na = digits_of(a, da), nb = digits_of(b, db);
    for (int i = 0; i < na && i < nb; i++)
        if (da[i] != db[i]) return da[i] < db[i];
    return na < nb;
}
template <int N>
SCLBM_HD constexpr int name_order(int i) {
    for (int j = 0; j < N; j++) {
        int rank = 0;
        for (int k = 0; k < N; k++) rank += name_less(k, j) ? 1 : 0;
        if (rank == i) return j;
    }
    return 0;
}

// Nonzero pattern of the exact noise operator (bit k of m[q]: coef[q][k] != 0),
// fixed by the lattice; the single-pass kernel skips the other terms.  A table
// with entries outside it (a reference kernel's literals carry 1e-17 residues)
// runs the dense two-pass kernel.  tests/test_gross.py checks these against
// the operator builder.
template <class L>
struct NoiseMask;
template <>
struct NoiseMask<D2Q9> {
    SCLBM_HD static constexpr unsigned m(int q) {
        constexpr unsigned t[9] = {0x25, 0x35, 0x2d, 0x35, 0x2d, 0x3f, 0x3f, 0x3f, 0x3f};
        return t[q];
    }
};
template <>
struct NoiseMask<D3Q19> {
    SCLBM_HD static constexpr unsigned m(int q) {
        constexpr unsigned t[19] = {0x7029, 0x3329, 0x7869, 0x3329, 0x7869, 0x74a9, 0x74a9, 0x116b, 0x116b, 0x116b,
                                    0x116b, 0x33ad, 0x33ad, 0x33ad, 0x33ad, 0x7cf9, 0x7cf9, 0x7cf9, 0x7cf9};
        return t[q];
    }
};

template <class L, class Real>
struct NoiseParams {
    static constexpr int NR = L::Q - L::D - 1;
    int kind;                 // CRNG_*
    int indep;                // 0: one generator per moment, 1: two
    Real m2var[NR];           // -2 var_k
    Real coef[L::Q][NR];      // noise population q = sum_k coef[q][k] Rm_k
};

SCLBM_HD uint64_t crng_next(int kind, uint64_t s) {
    if (kind == CRNG_MMIX) return s * 6364136223846793005ULL + 1442695040888963407ULL;
    if (kind == CRNG_NUMREC) return (uint32_t)((uint32_t)s * 1664525U + 1013904223U);
    const uint64_t w = 16807ULL * (uint32_t)s;
    uint32_t r = (uint32_t)((w & 0x7fffffffULL) + (w >> 31));
    if (r & 0x80000000U) r = (r & 0x7fffffffU) + 1U;
    return r;
}

// state / RANDMAX of the generator: 2^64 - 1 (which is 2^64 in double),
// 2^32 - 1, 2^31 - 1
template <class Real, bool STRICT>
__device__ __forceinline__ Real crng_uniform(int kind, uint64_t s) {
    if constexpr (std::is_same<Real, double>::value) {
        if (kind == CRNG_MMIX) return __dmul_rn(__ull2double_rn(s), 0x1p-64);
        const double m = kind == CRNG_NUMREC ? 4294967295.0 : 2147483647.0;
        return STRICT ? __ddiv_rn(__uint2double_rn((uint32_t)s), m) : __uint2double_rn((uint32_t)s) / m;
    } else {
        if (kind == CRNG_MMIX) return __ull2float_rn(s) * 0x1p-64f;
        const float r = kind == CRNG_NUMREC ? 0x1p-32f : 4.656612875245797e-10f;  // 1 / (2^31 - 1)
        return __uint2float_rn((uint32_t)s) * r;
    }
}

// sqrt(-2 var log(u0)) * cos(2 pi u1) + 0, TWOPI = 6.283185307179586 as the reference defines it.
// FP32 (a statistical path, not a parity one): the SFU's approximate log2,
// square root and cosine (relative errors ~1e-7..1e-6, far below the FP32
// storage noise), the cosine taken on [-pi, pi) as -cos(2 pi (u1 - 1/2)).
template <class Real, bool STRICT>
__device__ __forceinline__ Real box_muller(Real m2var, Real u0, Real u1) {
    if constexpr (std::is_same<Real, double>::value) {
        if (STRICT)
            return __dadd_rn(__dmul_rn(sqrt(__dmul_rn(m2var, log(u0))), cos(__dmul_rn(6.283185307179586, u1))), 0.0);
        return sqrt(m2var * log(u0)) * cos(6.283185307179586 * u1);
    } else {
        float l2, r, c;
        asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l2) : "f"(u0));
        const float x = (m2var * 0.6931471805599453f) * l2;  // m2var ln(u0) >= 0
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        asm("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(6.283185307179586f * (u1 - 0.5f)));
        return -r * c;
    }
}

// A cell's generator states are loaded all at once (one memory latency per
// cell, issued before the force so that its gathers overlap it), advanced in
// registers and stored back: st[s] = seeds[s*V + g] for s < NR, or < 2 NR
// with two generators per moment.
// I: the offset type (int where streams x V < 2^31, checked on the host)
template <class L, class T, class I = int64_t>
__device__ __forceinline__ void noise_load(int indep, const T *__restrict__ seeds, int64_t V, int64_t g, T *st) {
    constexpr int NR = L::Q - L::D - 1;
    const T *b = seeds + g;
    const I v = (I)V;
#pragma unroll
    for (int s = 0; s < NR; s++) st[s] = b[s * v];
    if (indep) {
#pragma unroll
        for (int s = NR; s < 2 * NR; s++) st[s] = b[s * v];
    }
}
template <class L, class T, class I = int64_t>
__device__ __forceinline__ void noise_store(int indep, T *__restrict__ seeds, int64_t V, int64_t g, const T *st) {
    constexpr int NR = L::Q - L::D - 1;
    T *b = seeds + g;
    const I v = (I)V;
#pragma unroll
    for (int s = 0; s < NR; s++) b[s * v] = st[s];
    if (indep) {
#pragma unroll
        for (int s = NR; s < 2 * NR; s++) b[s * v] = st[s];
    }
}

// u0 = 0 (a generator state of 0: NUMREC reaches it once in 2^32 draws of a
// stream, MMIX once in 2^64) would make log(u0) infinite and, in the
// reference, the cell's populations with it; here that draw takes the
// generator's smallest positive uniform (the value of state 1).  The stored
// state and every other draw are unchanged.
template <class T>
__device__ __forceinline__ T nonzero_state(T a) {
    return a == 0 ? T(1) : a;
}

// advance the states and form the random moments.  KIND (a CRNG_* value, or 0
// for z.kind at run time): with the generator known at compile time only its
// own update and conversion are emitted, instead of all three generators'
// updates and a run-time selection among them
template <class L, class Real, bool STRICT, class T, int KIND = 0>
__device__ __forceinline__ void noise_compute(const NoiseParams<L, Real> &z, int indep, T *st, Real *rm) {
    constexpr int NR = NoiseParams<L, Real>::NR;
    const int kind = KIND ? KIND : z.kind;
    if (indep) {
#pragma unroll
        for (int k = 0; k < NR; k++) {
            const T a = (T)crng_next(kind, st[2 * k]), b = (T)crng_next(kind, st[2 * k + 1]);
            st[2 * k] = a;
            st[2 * k + 1] = b;
            rm[k] = box_muller<Real, STRICT>(z.m2var[k], crng_uniform<Real, STRICT>(kind, nonzero_state(a)),
                                             crng_uniform<Real, STRICT>(kind, b));
        }
    } else {
#pragma unroll
        for (int k = 0; k < NR; k++) {
            const T a = (T)crng_next(kind, st[k]);
            const T b = (T)crng_next(kind, a);
            st[k] = b;
            rm[k] = box_muller<Real, STRICT>(z.m2var[k], crng_uniform<Real, STRICT>(kind, nonzero_state(a)),
                                             crng_uniform<Real, STRICT>(kind, b));
        }
    }
}

// out[q] += sum_k coef[q][k] Rm_k, term by term in the reference's print order
// (a pack expansion, so every moment index is a compile-time constant)
template <int NR, int I, class Real, bool STRICT>
__device__ __forceinline__ void add_noise_term(const Real *coef, const Real *rm, Real &acc) {
    constexpr int k = name_order<NR>(I);
    if constexpr (STRICT) acc = __dadd_rn(acc, __dmul_rn(coef[k], rm[k]));
    else acc = fma(coef[k], rm[k], acc);
}
template <int NR, class Real, bool STRICT, int... I>
__device__ __forceinline__ void add_noise_terms(const Real *coef, const Real *rm, Real &acc,
                                                std::integer_sequence<int, I...>) {
    (add_noise_term<NR, I, Real, STRICT>(coef, rm, acc), ...);
}
// FP32 single pass: the noise of one population, sum_k coef[k] Rm_k from the
// moments in registers, terms outside the lattice's nonzero pattern skipped
// (mask a constant after unrolling), in the reference's print order
template <int NR, int I>
__device__ __forceinline__ void noise_term_masked(unsigned mask, const float *coef, const float *rm, float &acc) {
    constexpr int k = name_order<NR>(I);
    if ((mask >> k) & 1u) acc = fmaf(coef[k], rm[k], acc);
}
template <int NR, int... I>
__device__ __forceinline__ float noise_sum_masked(unsigned mask, const float *coef, const float *rm,
                                                  std::integer_sequence<int, I...>) {
    float acc = 0.f;
    (noise_term_masked<NR, I>(mask, coef, rm, acc), ...);
    return acc;
}
template <class L, class Real, bool STRICT>
__device__ __forceinline__ void add_noise(const NoiseParams<L, Real> &z, const Real *rm, Real *out) {
    constexpr int NR = NoiseParams<L, Real>::NR;
#pragma unroll
    for (int q = 0; q < L::Q; q++)
        add_noise_terms<NR, Real, STRICT>(z.coef[q], rm, out[q], std::make_integer_sequence<int, NR>{});
}

// FP32: four CTAs of 128 threads per SM (at most 128 registers a thread), or
// the batched generator-state loads would take the whole register file; FP64
// (bound by the FP64 rate, not by occupancy): two, so nothing spills
template <class L, class S, class Real, bool STRICT, class T>
__global__ void __launch_bounds__(128, std::is_same<Real, float>::value ? 4 : 2) k_fcs_noise(const Real *__restrict__ pop, Real *__restrict__ pop_out,
                                                  const Real *__restrict__ dn, const Real *__restrict__ psi,
                                                  T *__restrict__ seeds,
                                                  const __grid_constant__ StepParams<L, S, Real> p,
                                                  const __grid_constant__ NoiseParams<L, Real> z) {
    constexpr int D = L::D, Q = L::Q, NR = NoiseParams<L, Real>::NR;
    const int64_t V = p.geo.V;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        Cell<D> c;
        cell_of<D>(g, p.geo.L, c);
        Real f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = __ldg(pop + (int64_t)q * V + g);
        T st[2 * NR];
        noise_load<L, T>(z.indep, seeds, V, g, st);
        const Real d = __ldg(dn + g);
        const Real n = p.rho0 + d;
        Real F[D], u[D];
        force_velocity<L, S, Real, STRICT>(psi, c, g, p, f, n, F, u);
        Real out[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) collide_cell<L, S, false, Real, STRICT>(f, d, n, u, F, q, p, out[q]);
        Real rm[NR];
        noise_compute<L, Real, STRICT, T>(z, z.indep, st, rm);
        noise_store<L, T>(z.indep, seeds, V, g, st);
        add_noise<L, Real, STRICT>(z, rm, out);
        if constexpr (std::is_same<Real, float>::value) {
            // FP32 storage: rest population from mass conservation (the noise carries no mass)
            Real rest = d;
#pragma unroll
            for (int q = 1; q < Q; q++) rest = __fsub_rn(rest, out[q]);
            out[0] = rest;
        }
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int64_t dst = index_at<D>(c, L::xi(q, 0), L::xi(q, 1), D == 3 ? L::xi(q, 2) : 0, p.geo.L);
            pop_out[(int64_t)q * V + dst] = out[q];
        }
    }
}

}  // namespace sclbm
