// Per-lattice observables of a batch (FP32-shifted storage, FP64 reductions):
// density/psi of every active lattice, then the Guo-shifted velocity with the
// convergence measure of CheckUConvergenceSCMP (idpy/LBM/MultiPhaseLoopChecks.py:96-163)
// per lattice: sum_cells sum_d |u - u_old|, max |u|^2 and the mass.  Grid:
// (blocks per lattice, lattices); per-block FP64 partials, summed on the host
// in a fixed order.
#pragma once

#include "fused.cuh"

namespace sclbm {

constexpr int BATCH_THREADS = 256;
constexpr int BATCH_NV = 3;  // sum |du|, max |u|^2, mass

template <class L>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_density(const float *__restrict__ pop, float *__restrict__ dn,
                                                                float *__restrict__ psi,
                                                                const BatchInst *__restrict__ inst, const int Vtot,
                                                                const int psi_kind) {
    const BatchInst I = inst[blockIdx.y];
    if (!I.active) return;
    const int V = I.Lx * I.Ly * I.Lz;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < V; g += gridDim.x * blockDim.x) {
        const float *src = pop + I.base + g;
        float s = src[lex_q<L::Q>(0) * Vtot];
#pragma unroll
        for (int i = 1; i < L::Q; i++) s += src[lex_q<L::Q>(i) * Vtot];
        dn[I.base + g] = s;
        psi[I.base + g] = psi_fast(psi_kind, I.rho0 + s);
    }
}

__device__ __forceinline__ void batch_block_reduce(double (&v)[BATCH_NV], double *out) {
    __shared__ double sh[BATCH_NV][BATCH_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < BATCH_NV; i++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double w = __shfl_down_sync(0xffffffffu, v[i], o);
            v[i] = i == 1 ? fmax(v[i], w) : v[i] + w;
        }
        if (lane == 0) sh[i][wid] = v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r[BATCH_NV] = {0.0, 0.0, 0.0};
        for (int w = 0; w < BATCH_THREADS / 32; w++) {
            r[0] += sh[0][w];
            r[1] = fmax(r[1], sh[1][w]);
            r[2] += sh[2][w];
        }
        for (int i = 0; i < BATCH_NV; i++) out[i] = r[i];
    }
}

// equilibrium at rest of every lattice from its density deviation:
// f_q - w_q rho0 = w_q (n - rho0)
template <class L>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_init(float *__restrict__ pop, const float *__restrict__ dn,
                                                             const BatchInst *__restrict__ inst, const int Vtot,
                                                             const float *__restrict__ wq) {
    const BatchInst I = inst[blockIdx.y];
    const int V = I.Lx * I.Ly * I.Lz;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < V; g += gridDim.x * blockDim.x) {
        const float d = dn[I.base + g];
#pragma unroll
        for (int q = 0; q < L::Q; q++) pop[q * Vtot + I.base + g] = wq[q] * d;
    }
}

template <class L, class S>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_moments(const float *__restrict__ pop, const float *__restrict__ dn,
                                                                const float *__restrict__ psi, float *__restrict__ u_old,
                                                                const __grid_constant__ StepParams<L, S, float> p,
                                                                const BatchInst *__restrict__ inst, const int Vtot,
                                                                double *partials) {
    constexpr int D = L::D, Q = L::Q;
    const BatchInst I = inst[blockIdx.y];
    double v[BATCH_NV] = {0.0, 0.0, 0.0};
    if (I.active) {
        const int V = I.Lx * I.Ly * I.Lz;
        for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < V; g += gridDim.x * blockDim.x) {
            const int x = g % I.Lx, r = g / I.Lx, y = r % I.Ly, z = r / I.Ly;
            float F[D];
#pragma unroll
            for (int c = 0; c < D; c++) F[c] = 0.f;
#pragma unroll
            for (int a = 0; a < S::QE; a++) {
                const int X = wrapc(x + S::e(a, 0), I.Lx), Y = wrapc(y + S::e(a, 1), I.Ly);
                const int Z = D == 3 ? wrapc(z + S::e(a, 2), I.Lz) : 0;
                const float ps = psi[I.base + X + I.Lx * (Y + I.Ly * Z)];
#pragma unroll
                for (int c = 0; c < D; c++)
                    if (S::e(a, c) != 0) F[c] = fmaf(p.sw[a][c], ps, F[c]);
            }
            const float sc = I.neg_g * psi[I.base + g];
#pragma unroll
            for (int c = 0; c < D; c++) F[c] *= sc;
            float f[Q];
#pragma unroll
            for (int q = 0; q < Q; q++) f[q] = pop[q * Vtot + I.base + g];
            const float d = dn[I.base + g];
            const float n = I.rho0 + d;
            float u[D];
            velocity<L, float>(f, n, F, u);
            double du = 0.0, u2 = 0.0;
#pragma unroll
            for (int c = 0; c < D; c++) {
                float &old = u_old[c * Vtot + I.base + g];
                du += fabs((double)u[c] - (double)old);
                u2 += (double)u[c] * (double)u[c];
                old = u[c];
            }
            v[0] += du;
            v[1] = fmax(v[1], u2);
            v[2] += (double)n;
        }
    }
    batch_block_reduce(v, partials + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * BATCH_NV);
}

// Exact mass of every active lattice, rho0 V + sum of its stored populations
// (FP64 sums of the FP32 values; slot 2 of the partials).  The density that
// k_batch_moments sums is an FP32 sum per cell, whose rounding would bias a
// mass correction.
template <class L>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_mass(const float *__restrict__ pop,
                                                             const BatchInst *__restrict__ inst, const int Vtot,
                                                             double *partials) {
    const BatchInst I = inst[blockIdx.y];
    double v[BATCH_NV] = {0.0, 0.0, 0.0};
    if (I.active) {
        const int V = I.Lx * I.Ly * I.Lz;
        for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < V; g += gridDim.x * blockDim.x) {
            double s = (double)I.rho0;
#pragma unroll
            for (int q = 0; q < L::Q; q++) s += (double)pop[q * Vtot + I.base + g];
            v[2] += s;
        }
    }
    batch_block_reduce(v, partials + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * BATCH_NV);
}

// add delta[i] to the rest population (q = 0) of every cell of active lattice i
// (a uniform correction; one proportional to |n - rho0| per cell, where FP32
// rounding loses the mass, made the Laplace pressures of the batched sweep
// agree less with the FP64 runs: median 9e-5 against 2e-5)
template <class L>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_add_rest(float *__restrict__ pop,
                                                                 const BatchInst *__restrict__ inst, const int Vtot,
                                                                 const float *__restrict__ delta) {
    const BatchInst I = inst[blockIdx.y];
    const float dl = delta[blockIdx.y];
    if (!I.active || dl == 0.f) return;
    const int V = I.Lx * I.Ly * I.Lz;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < V; g += gridDim.x * blockDim.x) pop[I.base + g] += dl;
}

// density (FP64 sum) at the centre cell (L_d / 2 in every dimension) and at
// the last cell of each active lattice: the two values DeltaPLaplace reads
// (K_NInNOut, idpy/LBM/LBMKernels.py:506-523).  One warp per lattice.
template <class L>
__global__ void __launch_bounds__(32) k_batch_probe(const float *__restrict__ pop, const BatchInst *__restrict__ inst,
                                                   const int Vtot, double *out, const int rad) {
    // density at the centre cell and at the last cell (DeltaPLaplace's two
    // probes), each the FP64 mean over the cube of side 2 rad + 1 about the
    // cell (periodic); rad = 0 is the single cell.  One warp per lattice,
    // cells taken in a fixed order by fixed lanes (reproducible sums).
    const BatchInst I = inst[blockIdx.x];
    if (!I.active) return;
    constexpr int D = L::D;
    const int side = 2 * rad + 1, cells = D == 3 ? side * side * side : side * side;
    const int Ls[3] = {I.Lx, I.Ly, D == 3 ? I.Lz : 1};
    const int cen[2][3] = {{I.Lx / 2, I.Ly / 2, D == 3 ? I.Lz / 2 : 0}, {I.Lx - 1, I.Ly - 1, D == 3 ? I.Lz - 1 : 0}};
    for (int which = 0; which < 2; which++) {
        double acc = 0.0;
        for (int t = threadIdx.x; t < cells; t += 32) {
            int o[3] = {t % side - rad, (t / side) % side - rad, D == 3 ? t / (side * side) - rad : 0};
            int idx = 0, stride = 1;
            for (int d = 0; d < 3; d++) {
                int v = (cen[which][d] + o[d]) % Ls[d];
                if (v < 0) v += Ls[d];
                idx += v * stride;
                stride *= Ls[d];
            }
            double n = 0.0;
#pragma unroll
            for (int q = 0; q < L::Q; q++) n += (double)pop[(int64_t)q * Vtot + I.base + idx];
            acc += n;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (threadIdx.x == 0) out[2 * blockIdx.x + which] = (double)I.rho0 + acc / cells;
    }
}

}  // namespace sclbm
