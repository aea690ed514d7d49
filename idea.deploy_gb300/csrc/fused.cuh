// Single-pass FP32 step: each CTA owns a tile of the lattice in the leading
// dimensions (x, or x-y in 3D) and marches along the last dimension (y in 2D,
// z in 3D) over a chunk of planes.  For every new plane it reduces the Q
// populations of the tile plus an R-wide halo to n and psi (psi kept in a
// shared-memory ring of 2R+1 planes), so the E4/E6/E8 force stencil reads
// psi from shared memory and the populations make one trip from HBM per step
// (the halo re-reads are served by L2: neighbouring tiles march the same
// planes at the same time).  Then each thread collides its interior cell and
// push-streams the Q results (as the reference, idpy/LBM/Collisions.py:383-561).
//
// Storage: FP32 deviations g_q = f_q - w_q rho0.  The rest population is set
// from mass conservation, g*_0 = dn - sum_{q>0} g*_q, so FP32 rounding of the
// collision coefficients cannot drift the total mass.
#pragma once

#include "kernels.cuh"

namespace sclbm {

template <class L, class S>
struct FusedShape {
    static constexpr int D = L::D;
    static constexpr int R = S::R;
    static constexpr int TX = D == 3 ? 32 : 256;     // tile width in x
    static constexpr int TY = D == 3 ? 8 : 1;        // tile height in y (3D)
    static constexpr int NT = TX * TY;               // threads = interior cells per plane
    static constexpr int HX = TX + 2 * R;            // halo tile width
    static constexpr int HY = D == 3 ? TY + 2 * R : 1;
    static constexpr int HC = HX * HY;               // halo cells per plane
    static constexpr int RING = 2 * R + 1;           // psi planes kept
    static constexpr int SMEM = RING * HC * 4;       // bytes of the psi ring
};

struct FusedGeom {
    int L[3];
    int64_t V;
    int tiles_x, tiles_y, chunks, chunk;  // work decomposition
    int items;
};

__device__ __forceinline__ int wrapm(int x, int L) {
    int r = x % L;
    return r < 0 ? r + L : r;
}

template <class L, class S, bool MRT>
__global__ void __launch_bounds__(FusedShape<L, S>::NT, 2)
    k_fused(const float *__restrict__ pop, float *__restrict__ pop_out, const __grid_constant__ StepParams<L, S, float> p,
            const FusedGeom fg) {
    using SH = FusedShape<L, S>;
    constexpr int D = L::D, Q = L::Q, R = SH::R, HX = SH::HX, HC = SH::HC, NT = SH::NT, RING = SH::RING;
    extern __shared__ float ring[];  // [RING][HC]
    const int tid = threadIdx.x;
    const int64_t V = fg.V;
    const int Lx = fg.L[0], Ly = fg.L[1], Lz = fg.L[2];
    const int Lm = D == 3 ? Lz : Ly;  // marching extent
    const int tx = tid % SH::TX, ty = D == 3 ? tid / SH::TX : 0;

    for (int item = blockIdx.x; item < fg.items; item += gridDim.x) {
        const int ix = item % fg.tiles_x;
        const int rest = item / fg.tiles_x;
        const int iy = D == 3 ? rest % fg.tiles_y : 0;
        const int ic = D == 3 ? rest / fg.tiles_y : rest;
        const int x0 = ix * SH::TX, y0 = iy * SH::TY;
        const int m0 = ic * fg.chunk, m1 = min(m0 + fg.chunk, Lm);

        // n and psi of the halo tile of plane m into its ring slot
        auto psi_plane = [&](int m) {
            float *slot = ring + wrapm(m, RING) * HC;
            const int gm = wrapm(m, Lm);
            for (int c = tid; c < HC; c += NT) {
                const int hx = c % HX, hy = c / HX;
                const int gx = wrapm(x0 - R + hx, Lx);
                int64_t g;
                if (D == 3) g = gx + (int64_t)Lx * (wrapm(y0 - R + hy, Ly) + (int64_t)Ly * gm);
                else g = gx + (int64_t)Lx * gm;
                float s = __ldg(pop + (int64_t)lex_q<Q>(0) * V + g);
#pragma unroll
                for (int i = 1; i < Q; i++) s += __ldg(pop + (int64_t)lex_q<Q>(i) * V + g);
                slot[c] = psi_of<float>(p.psi_kind, p.rho0 + s);
            }
        };

        for (int m = m0 - R; m < m0 + R; m++) psi_plane(m);
        for (int m = m0; m < m1; m++) {
            psi_plane(m + R);
            __syncthreads();
            const int x = x0 + tx, y = D == 3 ? y0 + ty : m;
            const bool inside = x < Lx && (D == 2 || y < Ly);
            if (inside) {
                const int z = D == 3 ? m : 0;
                const int64_t g = D == 3 ? x + (int64_t)Lx * (y + (int64_t)Ly * z) : x + (int64_t)Lx * y;
                float f[Q];
#pragma unroll
                for (int q = 0; q < Q; q++) f[q] = __ldg(pop + (int64_t)q * V + g);
                float d = f[lex_q<Q>(0)];
#pragma unroll
                for (int i = 1; i < Q; i++) d += f[lex_q<Q>(i)];
                // Shan-Chen force from the psi ring
                float F[D];
#pragma unroll
                for (int a = 0; a < D; a++) F[a] = 0.f;
#pragma unroll
                for (int a = 0; a < S::QE; a++) {
                    const int em = D == 3 ? S::e(a, 2) : S::e(a, 1);
                    const int ey = D == 3 ? S::e(a, 1) : 0;
                    const int row = D == 3 ? (ty + R + ey) : 0;  // 2D: one halo row per plane
                    const float ps = ring[wrapm(m + em, RING) * HC + row * HX + (tx + R + S::e(a, 0))];
#pragma unroll
                    for (int c = 0; c < D; c++)
                        if (S::e(a, c) != 0) F[c] = fmaf(p.sw[a][c], ps, F[c]);
                }
                const float ps0 = ring[wrapm(m, RING) * HC + (D == 3 ? (ty + R) * HX : 0) + (tx + R)];
                const float sc = p.neg_g * ps0;
#pragma unroll
                for (int c = 0; c < D; c++) F[c] *= sc;
                const float n = p.rho0 + d;
                float u[D];
                velocity<L, float>(f, n, F, u);
                float out[Q];
                float rest = d;
#pragma unroll
                for (int q = 1; q < Q; q++) {
                    collide_cell<L, S, MRT, float, false>(f, d, n, u, F, q, p, out[q]);
                    rest -= out[q];
                }
                out[0] = rest;
                // push stream
                int xs[3], ys[3], zs[3];
#pragma unroll
                for (int o = -1; o <= 1; o++) {
                    xs[o + 1] = wrapc(x + o, Lx);
                    ys[o + 1] = wrapc(y + o, Ly);
                    zs[o + 1] = D == 3 ? wrapc(z + o, Lz) : 0;
                }
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    const int X = xs[L::xi(q, 0) + 1], Y = ys[L::xi(q, 1) + 1];
                    int64_t dst = X + (int64_t)Lx * Y;
                    if (D == 3) dst += (int64_t)Lx * Ly * zs[L::xi(q, 2) + 1];
                    pop_out[(int64_t)q * V + dst] = out[q];
                }
            }
            __syncthreads();
        }
    }
}

}  // namespace sclbm
