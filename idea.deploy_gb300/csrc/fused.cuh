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
//
// Index arithmetic is kept off the critical path: cell offsets are 32-bit
// (V < 2^31, checked on the host), the halo cells a thread reduces and the
// wrapped neighbour rows / planes are computed once per tile or plane, and
// every shared-memory stencil read has a compile-time offset from one of the
// 2R+1 per-plane slot bases.
#pragma once

#include <cuda.h>  // CUtensorMap (the tensor maps are encoded on the host)

#include "kernels.cuh"
#include "noise.cuh"

namespace sclbm {

// Staging of the 3D single pass (bit flags; 0 = every load straight into registers):
//   STG_HALO_ASYNC  the halo pairs of plane m+R+1 are copied into this thread's
//                   own shared-memory slots with cp.async while plane m collides
//                   (each thread reads back only what it copied: no barrier)
//   STG_OWN_TMA     the tile's own populations of plane m+1 come in by one TMA
//                   box (x, y, plane, q) = (TX, TY, 1, Q) per plane, double
//                   buffered, completed on an mbarrier, while plane m collides
enum : int { STG_HALO_ASYNC = 1, STG_OWN_TMA = 2 };

// Tile shapes of the 3D paired single pass (BGK): index 0 is the default
// 32 x 8 (256 threads, four CTAs per SM); the others put wider rows (256 or
// 512 bytes of a population row per CTA, which the memory system serves
// better than 128-byte pieces) or more rows (a smaller halo share) in a CTA:
// 64 x 8 and 32 x 16 (512 threads, two CTAs per SM), 128 x 8 (1024 threads,
// one).  Every shape computes the same cells with the same arithmetic, so the
// results are bit-identical; the autotuner picks among them.
// Shape 4 is the default shape with streaming stores (st.global.cs: the
// pushed populations are not read again within the step, so they are marked
// evict-first and leave L2 to the halo lines that neighbouring tiles re-read).
// Shape 5 is the default shape with the per-plane __syncthreads replaced by
// an mbarrier per psi-ring slot: a thread arrives once it has written its psi
// values of a plane and waits only for the slot it is about to read, so warps
// may drift apart by up to two planes instead of meeting at every plane (the
// ring holds 2R+4 planes so that a slot is rewritten only after the slowest
// warp has left it).  The waits are bounded (an error flag for the host).
struct TileShape {
    int tx, ty, minb, cs, mb;
};
constexpr TileShape kTiles[] = {{32, 8, 4, 0, 0}, {64, 8, 2, 0, 0}, {32, 16, 2, 0, 0},
                                {128, 8, 1, 0, 0}, {32, 8, 4, 1, 0}, {32, 8, 4, 0, 1}};
constexpr int N_TILES = 6;

template <class L, class S, int TXp = 0, int TYp = 0>
struct FusedShape {
    static constexpr int D = L::D;
    static constexpr int R = S::R;
    static constexpr int TX = TXp ? TXp : (D == 3 ? 32 : 256);  // tile width in x
    static constexpr int TY = TYp ? TYp : (D == 3 ? 8 : 1);     // tile height in y (3D)
    static constexpr int NT = TX * TY;               // threads = interior cells per plane
    static constexpr int HX = TX + 2 * R;            // halo tile width
    static constexpr int HY = D == 3 ? TY + 2 * R : 1;
    static constexpr int HC = HX * HY;               // halo cells per plane
    static constexpr int HPT = (HC + NT - 1) / NT;   // halo cells per thread
    // psi planes kept: 2R+1 in use plus one being written, so one barrier per
    // plane suffices (the slot written for plane m+R held plane m-R-2)
    static constexpr int RING = 2 * R + 2;
    // floats of one plane's staged halo populations (2D only: see k_fused)
    static constexpr int STAGE = D == 2 ? HPT * L::Q * NT : 0;
    static constexpr int SMEM = (RING * HC + 2 * STAGE) * 4;  // psi ring + double-buffered stage
    // fluctuating step: plus each thread's noise of its current cell's Q - 1
    // moving populations
    static constexpr int NSMEM = SMEM + (L::Q - 1) * NT * 4;
    // walls: plus a ring of the halo planes' wall flags (bytes)
    static constexpr int WSMEM = SMEM + (RING * HC + 3) / 4 * 4;
    // staged variants (3D): halo-pair slots [Q][HSTR] float2, then two own
    // buffers [Q][TY][TX] float (128-byte aligned: TMA destinations) and their
    // two mbarriers
    static constexpr int NPAIR = (HX / 2) * HY;
    static constexpr int HSTR = (NPAIR + 31) / 32 * 32;
    static constexpr int RING_BYTES = RING * HC * 4;
    static constexpr int HALO_BYTES = L::Q * HSTR * 8;
    static constexpr int OWN_BOX_BYTES = L::Q * NT * 4;
    static constexpr int own_offset(int stg) {
        return ((RING_BYTES + ((stg & STG_HALO_ASYNC) ? HALO_BYTES : 0)) + 127) / 128 * 128;
    }
    // the mbarrier-ring variant: 2R+4 psi planes and one mbarrier per slot
    static constexpr int MB_RING = 2 * R + 4;
    static constexpr int MB_SMEM = MB_RING * HC * 4 + MB_RING * 8;
    static constexpr int stg_smem(int stg) {
        return (stg & STG_OWN_TMA) ? own_offset(stg) + 2 * OWN_BOX_BYTES + 16
                                   : RING_BYTES + ((stg & STG_HALO_ASYNC) ? HALO_BYTES : 0);
    }
};

// ---- PTX helpers of the staged variants ------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// box (c0, c1, c2, c3) of a 4D tensor map into shared memory, completing on bar
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}
// Bounded wait on an mbarrier phase: a TMA that never completes (it cannot,
// unless the tensor map or the byte count is wrong) must not hang the GPU.
// After MBAR_POLLS unsuccessful polls the wait gives up, records the failure in
// *err (read by the host after the launch) and the kernel runs on with the
// buffer as it is (no thread leaves the block's barriers); later waits of the
// launch then return at once.  An unsuccessful try_wait returns after ~4 us
// on a GB300 (measured by the bounded-wait self-test), so 2^18 polls give up
// after about a second.
constexpr int MBAR_POLLS = 1 << 18;
__device__ __forceinline__ void mbar_wait_bounded(uint64_t *bar, unsigned parity, int *err, bool &dead,
                                                  int polls = MBAR_POLLS) {
    if (dead) return;
    for (int i = 0; i < polls; i++)
        if (mbar_try_wait(bar, parity)) return;
    dead = true;
    if (err) atomicOr(err, 1);
}


__device__ __forceinline__ void cp_async4(float *smem, const float *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

struct FusedGeom {
    int L[3];
    int64_t V;
    int tiles_x, tiles_y, chunks, chunk;  // work decomposition
    int items;
    int pairs;  // 3D, even Lx and even halo radius: halo populations loaded two cells per load
    int stg;    // STG_* flags of the staged 3D variants (0: none)
    int tile;   // index into kTiles (3D paired BGK; 0: the default shape)
    int order;  // order of the work items over the grid (k_fused; 0 x, 1 chunk, 2 y fastest)
    int *err;   // device flag set by a staged variant whose bounded wait gave up
};

// FP32 pseudopotential with the fast hardware exp2/reciprocal (relative error
// ~1e-7, below the FP32 storage of the populations)
__device__ __forceinline__ float psi_fast(int kind, float n) {
    if (kind == PSI_EXP_INV) return __expf(-__fdividef(1.f, n));
    if (kind == PSI_ONE_MINUS_EXP) return 1.f - __expf(-n);
    return n;
}

__device__ __forceinline__ int wrapm(int x, int L) {
    int r = x % L;
    return r < 0 ? r + L : r;
}

// BGK + Guo collision of one cell in FP32-shifted variables (c2 = 1/3), factored:
//   g*_q = (1-w) g_q + w_q [ C0 + eu (a eu + b + c eF) + d eF ]
// eu = xi_q.u, eF = xi_q.F, C0 = w dn - 1.5 w n u^2 - 3 (1-w/2) u.F,
// a = 4.5 w n, b = 3 w n, c = 9 (1-w/2), d = 3 (1-w/2); the same operator as
// the expanded form (2nd-order Hermite equilibrium + Guo term, Collisions.py:163-185).
// A direction q and its opposite qb (eu and eF change sign) are made together:
// with t = a eu^2 + c eu eF (even in xi) and s = b eu + d eF (odd in xi),
//   g*_q = (1-w) g_q + w_q (C0 + t + s),  g*_qb = (1-w) g_qb + w_qb (C0 + t - s),
// so eu, eF, t and C0 + t are computed once for the two.
template <class L, class S>
__device__ __forceinline__ void bgk_pair_fp32(const float *f, const float *u, const float *F, int q, int qb,
                                              const StepParams<L, S, float> &p, float C0, float a, float b,
                                              float &out_q, float &out_qb) {
    constexpr int D = L::D;
    float eu = 0.f, eF = 0.f;
#pragma unroll
    for (int c = 0; c < D; c++) {
        if (L::xi(q, c) > 0) { eu += u[c]; eF += F[c]; }
        if (L::xi(q, c) < 0) { eu -= u[c]; eF -= F[c]; }
    }
    const float even = eu * fmaf(a, eu, p.fc * eF);
    const float odd = fmaf(b, eu, p.fd * eF);
    const float base = C0 + even;
    const float rq = p.wq[q] * (base + odd), rqb = p.wq[qb] * (base - odd);
    out_q = p.a_nonzero ? fmaf(p.A[q][q], f[q], rq) : rq;
    out_qb = p.a_nonzero ? fmaf(p.A[qb][qb], f[qb], rqb) : rqb;
}

// index of the force-stencil vector opposite to e_a, from a table the
// compiler builds once per stencil (a search per unrolled use would not fold)
template <class S>
struct OppositeE {
    int v[S::QE];
    constexpr OppositeE() : v() {
        for (int a = 0; a < S::QE; a++) {
            v[a] = a;
            for (int k = 0; k < S::QE; k++) {
                bool same = true;
                for (int d = 0; d < S::D; d++) same = same && (S::e(k, d) == -S::e(a, d));
                if (same) v[a] = k;
            }
        }
    }
};
template <class S>
SCLBM_HD constexpr int opposite_e(int a) {
    constexpr OppositeE<S> t{};
    return t.v[a];
}

// One work item: the tile (x0, y0) of one lattice, planes [m0, m1).  pop and
// pop_out point at the lattice's first cell, V is the distance between two
// populations of a cell (the lattice volume, or a batch's total volume).
// ST (not void): the fluctuating step (noise.cuh), generator states of type ST
// at seeds[s*V + cell].
// WALLS: wall flags (1 fluid, 0 wall; other values neither) and the psi the
// walls keep, as k_density_psi_walls + k_fcs_walls: n and psi of fluid cells
// only, the walls' psi elsewhere; non-fluid cells pass their populations on
// unchanged; a population pushed into a wall cell goes to the opposite
// population of its own cell (halfway bounce-back).  The halo planes' flags sit
// in a shared-memory ring beside the psi ring.
// PAIRS (3D, even radius R, even Lx): the halo reduction loads each
// population of two x-adjacent cells with one 8-byte load.  The halo row is
// TX + 2R cells wide and starts at an even x, so a row is (TX + 2R)/2 whole
// pairs that never straddle the periodic wrap; one thread reduces one pair
// ((TX/2 + R) * (TY + 2R) <= NT pairs per plane), which halves the halo load
// and address instructions of the scalar form (two cells per thread, the
// second re-read by threads that have none).  The sums run in the same order,
// so the results are bit-identical to the scalar form.
// STG (3D, PAIRS, no walls or noise): STG_* staging flags.  With STG_OWN_TMA
// the caller passes the input's tensor map, the two mbarriers, the running
// issue / wait counts of own-population boxes (k_issue-th box: buffer k & 1,
// phase (k >> 1) & 1, the same on every thread) and the error flag.
// error-free sum (Knuth's TwoSum): a + b = s + e exactly, s the rounded sum
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// EXACT_REST: the rest population balances the cell's mass with the rounding
// errors of the density sum and of the subtraction chain carried along
// (TwoSum), so that a cell's stored FP32 populations sum to its incoming ones
// up to one rounding of the rest population.  Without it the ~36 roundings
// per cell repeat in a near-steady state and drift the mass by ~1e-9 per
// step; the batched sweeps use it (their Laplace-pressure criterion sees that
// drift on large droplets).  The density used by the physics is unchanged.
template <class L, class S, bool MRT, class ST = void, bool WALLS = false, bool PAIRS = false, int STG = 0,
          int TXT = 0, int TYT = 0, bool EXACT_REST = false, bool CS = false, bool MB = false, int CRNG = 0>
__device__ __forceinline__ void fused_tile(const float *__restrict__ pop, float *__restrict__ pop_out, const int V,
                                           const int Lx, const int Ly, const int Lz, const int x0, const int y0,
                                           const int m0, const int m1, const float neg_g, const float rho0,
                                           const StepParams<L, S, float> &p, float *smem,
                                           ST *seeds = nullptr, const NoiseParams<L, float> *z = nullptr,
                                           const unsigned char *__restrict__ walls = nullptr,
                                           const float *__restrict__ psi_w = nullptr,
                                           const CUtensorMap *tmap = nullptr, uint64_t *bars = nullptr,
                                           unsigned *k_issue = nullptr, unsigned *k_wait = nullptr,
                                           int *err = nullptr, bool *dead = nullptr) {
    constexpr bool NOISE = !std::is_void<ST>::value;
    static_assert(STG == 0 || (PAIRS && !NOISE && !WALLS && L::D == 3), "staged variants: 3D paired halo loads");
    constexpr bool HALO_ASYNC = (STG & STG_HALO_ASYNC) != 0, OWN_TMA = (STG & STG_OWN_TMA) != 0;
    using SeedT = typename std::conditional<NOISE, ST, int>::type;
    using SH = FusedShape<L, S, TXT, TYT>;
    constexpr int D = L::D, Q = L::Q, R = SH::R, HX = SH::HX, HC = SH::HC, NT = SH::NT;
    constexpr int RING = MB ? SH::MB_RING : SH::RING;
    static_assert(!MB || (PAIRS && STG == 0 && !WALLS && std::is_void<ST>::value && D == 3), "mbarrier ring");
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + RING * HC);  // MB: one per ring slot
    float *ring = smem;  // psi ring [RING][HC], then (2D) 2 stage buffers [HPT][Q][NT]
    float *stage0 = smem + RING * HC;
    unsigned char *fring = reinterpret_cast<unsigned char *>(smem + RING * HC + 2 * SH::STAGE);  // WALLS
    const int tid = threadIdx.x;
    const int Lm = D == 3 ? Lz : Ly;       // marching extent
    const int PL = D == 3 ? Lx * Ly : Lx;  // cells per plane
    const int tx = tid % SH::TX, ty = D == 3 ? tid / SH::TX : 0;

    // in-plane offsets of the halo cells this thread reduces (fixed per tile)
    int hoff[SH::HPT];
#pragma unroll
    for (int k = 0; k < SH::HPT; k++) {
        const int c = tid + k * NT;
        const int hx = c % HX, hy = c / HX;
        const int gx = wrapm(x0 - R + hx, Lx);
        hoff[k] = D == 3 ? gx + Lx * wrapm(y0 - R + hy, Ly) : gx;
    }
    // PAIRS: in-plane offset of the (even) first cell of this thread's halo pair
    constexpr int HP = HX / 2, NPAIR = HP * SH::HY;
    static_assert(!PAIRS || (D == 3 && R % 2 == 0 && NPAIR <= NT && !WALLS), "paired halo loads");
    int hoffp = 0;
    if constexpr (PAIRS) {
        const int c = tid < NPAIR ? tid : 0;
        hoffp = wrapm(x0 - R + 2 * (c % HP), Lx) + Lx * wrapm(y0 - R + c / HP, Ly);
    }
    // interior cell of this thread and its wrapped neighbour columns / rows
    const int x = x0 + tx, y = D == 3 ? y0 + ty : 0;
    const bool in_tile = x < Lx && (D == 2 || y < Ly);
    int X3[3], Y3[3];
#pragma unroll
    for (int o = -1; o <= 1; o++) {
        X3[o + 1] = wrapc(x + o, Lx);
        Y3[o + 1] = D == 3 ? Lx * wrapc(y + o, Ly) : 0;
    }
    const int own_cell = X3[1] + Y3[1];

    // n and psi of plane m straight from global memory; every load is issued
    // before the first sum (threads without a second halo cell re-read their
    // first one and skip the store), so HPT*Q loads are in flight at once
    auto psi_plane = [&](int m) {
        float *slot = ring + wrapm(m, RING) * HC;
        const int poff = wrapm(m, Lm) * PL;
        if constexpr (PAIRS) {
            // halo cell c = 2*tid and 2*tid+1 of the plane (HX = 2*HP)
            if (tid < NPAIR) {
                const float2 *src = reinterpret_cast<const float2 *>(pop + (poff + hoffp));
                const int V2 = V >> 1;
                float2 w[Q];
#pragma unroll
                for (int q = 0; q < Q; q++) w[q] = __ldg(src + q * V2);
                float sx = w[lex_q<Q>(0)].x, sy = w[lex_q<Q>(0)].y;
#pragma unroll
                for (int i = 1; i < Q; i++) {
                    sx += w[lex_q<Q>(i)].x;
                    sy += w[lex_q<Q>(i)].y;
                }
                reinterpret_cast<float2 *>(slot)[tid] =
                    make_float2(psi_fast(p.psi_kind, rho0 + sx), psi_fast(p.psi_kind, rho0 + sy));
            }
        } else {
        float v[SH::HPT][Q];
#pragma unroll
        for (int k = 0; k < SH::HPT; k++) {
            const int c = tid + k * NT;
            const float *src = pop + (poff + (c < HC ? hoff[k] : hoff[0]));
#pragma unroll
            for (int q = 0; q < Q; q++) v[k][q] = __ldg(src + q * V);
        }
#pragma unroll
        for (int k = 0; k < SH::HPT; k++) {
            const int c = tid + k * NT;
            float s = v[k][lex_q<Q>(0)];
#pragma unroll
            for (int i = 1; i < Q; i++) s += v[k][lex_q<Q>(i)];
            if (k + 1 < SH::HPT || c < HC) {
                float ps = psi_fast(p.psi_kind, rho0 + s);
                if constexpr (WALLS) {
                    const int cell = poff + hoff[k];
                    const unsigned char fl = walls[cell];
                    fring[wrapm(m, RING) * HC + c] = fl;
                    if (fl != 1) ps = psi_w[cell];
                }
                slot[c] = ps;
            }
        }
        }
    };
    // asynchronous copy of this thread's halo populations of plane m into a stage buffer
    auto stage_issue = [&](int m) {
        float *st = stage0 + (m & 1) * SH::STAGE;
        const int poff = wrapm(m, Lm) * PL;
#pragma unroll
        for (int k = 0; k < SH::HPT; k++) {
            const int c = tid + k * NT;
            if (k + 1 < SH::HPT || c < HC) {
                const float *src = pop + (poff + hoff[k]);
#pragma unroll
                for (int q = 0; q < Q; q++) cp_async4(st + (k * Q + q) * NT + tid, src + q * V);
            }
        }
        cp_async_commit();
    };
    // n and psi of plane m from the stage (each thread reads back only its own copies)
    auto stage_reduce = [&](int m) {
        const float *st = stage0 + (m & 1) * SH::STAGE;
        float *slot = ring + wrapm(m, RING) * HC;
        const int poff = wrapm(m, Lm) * PL;
#pragma unroll
        for (int k = 0; k < SH::HPT; k++) {
            const int c = tid + k * NT;
            if (k + 1 < SH::HPT || c < HC) {
                float s = st[(k * Q + lex_q<Q>(0)) * NT + tid];
#pragma unroll
                for (int i = 1; i < Q; i++) s += st[(k * Q + lex_q<Q>(i)) * NT + tid];
                float ps = psi_fast(p.psi_kind, rho0 + s);
                if constexpr (WALLS) {
                    const int cell = poff + hoff[k];
                    const unsigned char fl = walls[cell];
                    fring[wrapm(m, RING) * HC + c] = fl;
                    if (fl != 1) ps = psi_w[cell];
                }
                slot[c] = ps;
            }
        }
    };

    // STG_HALO_ASYNC: this thread's halo pair of plane m copied into its own
    // slots hst[q*HSTR + tid] (issued one plane ahead), reduced from there
    float2 *hst = reinterpret_cast<float2 *>(smem + RING * HC);
    auto halo_issue = [&](int m) {
        if constexpr (HALO_ASYNC) {
            if (tid < NPAIR) {
                const float2 *src = reinterpret_cast<const float2 *>(pop + (wrapm(m, Lm) * PL + hoffp));
                const int V2 = V >> 1;
#pragma unroll
                for (int q = 0; q < Q; q++) cp_async8(hst + q * SH::HSTR + tid, src + q * V2);
            }
            cp_async_commit();
        }
    };
    auto halo_reduce = [&](int m) {
        if constexpr (HALO_ASYNC) {
            cp_async_wait<0>();
            if (tid < NPAIR) {
                float2 w[Q];
#pragma unroll
                for (int q = 0; q < Q; q++) w[q] = hst[q * SH::HSTR + tid];
                float sx = w[lex_q<Q>(0)].x, sy = w[lex_q<Q>(0)].y;
#pragma unroll
                for (int i = 1; i < Q; i++) {
                    sx += w[lex_q<Q>(i)].x;
                    sy += w[lex_q<Q>(i)].y;
                }
                // the store needs every value read back, so the next cp.async
                // into these slots (issued after it) cannot overtake the reads
                reinterpret_cast<float2 *>(ring + wrapm(m, RING) * HC)[tid] =
                    make_float2(psi_fast(p.psi_kind, rho0 + sx), psi_fast(p.psi_kind, rho0 + sy));
            }
        }
    };
    // STG_OWN_TMA: the tile's populations of plane m, box (x0, y0, plane, 0),
    // into own buffer b (thread 0 issues)
    float *own = reinterpret_cast<float *>(reinterpret_cast<char *>(smem) + SH::own_offset(STG));
    auto own_issue = [&](int m) {
        if constexpr (OWN_TMA) {
            const int b = *k_issue & 1;
            if (tid == 0) {
                mbar_expect_tx(&bars[b], SH::OWN_BOX_BYTES);
                tma_load_4d(own + b * (SH::OWN_BOX_BYTES / 4), tmap, &bars[b], x0, y0, wrapm(m, Lm), 0);
            }
            (*k_issue)++;
        }
    };

    // 2D: the halo of plane m+R+1 is prefetched with cp.async during plane m;
    // 3D: the halo (1.7x the tile) is reduced straight from L2 and the
    // thread's own populations of plane m are loaded first, so both sets of
    // loads are in flight together
    constexpr bool STAGED = D == 2;
    __syncthreads();  // the previous item's readers are done with the ring (and the own buffers)
    if constexpr (MB) {
        // fresh phases for this item: every arrival of the previous item completed its phase
        if (tid == 0)
            for (int k = 0; k < RING; k++) {
                mbar_inval(&mbar[k]);
                mbar_init(&mbar[k], NT);
            }
        __syncthreads();
    }
    own_issue(m0);
    if constexpr (STAGED) {
        // 2D: the preamble's planes through the two stage buffers, the next
        // plane's copy in flight while this one is reduced (each thread reads
        // back only its own copies, so no barrier between a reduce and the
        // copy that reuses the buffer); same sums as psi_plane
        stage_issue(m0 - R);
        for (int m = m0 - R; m < m0 + R; m++) {
            if (m + 1 < m0 + R) {
                stage_issue(m + 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            stage_reduce(m);
        }
    } else {
        for (int m = m0 - R; m < m0 + R; m++) psi_plane(m);
    }
    if (STAGED) stage_issue(m0 + R);
    halo_issue(m0 + R);
    if constexpr (MB) {
        psi_plane(m0 + R);  // one plane ahead; the main loop computes m+R+1
        __syncthreads();
    }
    // 2D: the thread's own populations of plane m+1 are loaded while plane m
    // is computed (Q more registers), so their latency overlaps a whole plane
    // instead of the short stage reduction before the force needs them
    float fa[STAGED ? Q : 1];
    if constexpr (STAGED) {
        if (in_tile) {
#pragma unroll
            for (int q = 0; q < Q; q++) fa[q] = __ldg(pop + (own_cell + m0 * Lx + q * V));
        }
    }
    for (int m = m0; m < m1; m++) {
        int Z3[3];
#pragma unroll
        for (int o = -1; o <= 1; o++) Z3[o + 1] = D == 3 ? wrapc(m + o, Lm) * PL : wrapc(m + o, Lm) * Lx;
        const int g = own_cell + Z3[1];
        float f[Q];
        constexpr int NR = NoiseParams<L, float>::NR;
        SeedT st[NOISE ? NR : 1];
        if (in_tile && !OWN_TMA) {
            if constexpr (STAGED) {
#pragma unroll
                for (int q = 0; q < Q; q++) f[q] = fa[q];
                if (m + 1 < m1) {
#pragma unroll
                    for (int q = 0; q < Q; q++) fa[q] = __ldg(pop + (own_cell + (m + 1) * Lx + q * V));
                }
            } else {
#pragma unroll
                for (int q = 0; q < Q; q++) f[q] = __ldg(pop + (g + q * V));
            }
            // generator states with the populations: their loads overlap the psi plane
            // (one generator per moment: the two-generator mode runs the two-pass kernel)
            if constexpr (NOISE) noise_load<L, SeedT, int>(0, seeds, (int64_t)V, (int64_t)g, st);
        }
        if (STAGED) {
            if (m + 1 < m1) {
                stage_issue(m + R + 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            stage_reduce(m + R);
        } else if (HALO_ASYNC) {
            halo_reduce(m + R);
            if (m + 1 < m1) halo_issue(m + R + 1);
        } else if (MB) {
            if (m + 1 < m1) {
                psi_plane(m + R + 1);
                mbar_arrive(&mbar[wrapm(m + R + 1, RING)]);
            }
        } else {
            psi_plane(m + R);
        }
        if constexpr (MB) {
            // plane m+R was written in the previous iteration (or the preamble);
            // its slot's k-th main-loop use has phase k & 1
            if (m > m0) mbar_wait_bounded(&mbar[wrapm(m + R, RING)], ((m - m0 - 1) / RING) & 1, err, *dead);
        } else {
            __syncthreads();
        }
        if constexpr (OWN_TMA) {
            // buffer of plane m+1 was last read for plane m-1, before the barrier
            if (m + 1 < m1) own_issue(m + 1);
            const unsigned k = (*k_wait)++;
            const int b = k & 1;
            mbar_wait_bounded(&bars[b], (k >> 1) & 1, err, *dead);
            if (in_tile) {
                const float *ob = own + b * (SH::OWN_BOX_BYTES / 4) + tid;
#pragma unroll
                for (int q = 0; q < Q; q++) f[q] = ob[q * NT];
            }
        }
        if (in_tile) {
            // slot bases of planes m-R .. m+R, offset to this thread's halo position
            const float *sb[RING];
#pragma unroll
            for (int k = 0; k < RING; k++) sb[k] = ring + wrapm(m + k - R, RING) * HC + ty * HX + tx;
            // flags of planes m-1, m, m+1 at this thread's halo position
            const unsigned char *fb[3] = {nullptr, nullptr, nullptr};
            bool fluid = true;  // a non-fluid cell passes its populations on unchanged
            if constexpr (WALLS) {
#pragma unroll
                for (int o = 0; o < 3; o++)
                    fb[o] = fring + wrapm(m + o - 1, RING) * HC + ty * HX + tx + (D == 3 ? R * HX : 0) + R;
                fluid = fb[1][0] == 1;
            }
            // the cell's noise per moving population into this thread's
            // shared-memory slots (the states and moments die here; the
            // collision adds its population's noise back with one load)
            float *nzs = smem + SH::RING * SH::HC + 2 * SH::STAGE + tid;
            if constexpr (NOISE) {
                float rm[NR];
                noise_compute<L, float, false, SeedT, CRNG>(*z, 0, st, rm);
                noise_store<L, SeedT, int>(0, seeds, (int64_t)V, (int64_t)g, st);
#pragma unroll
                for (int q = 1; q < Q; q++)
                    nzs[(q - 1) * NT] = noise_sum_masked<NR>(NoiseMask<L>::m(q), z->coef[q], rm,
                                                             std::make_integer_sequence<int, NR>{});
            }
            if (!fluid) {
#pragma unroll
                for (int q = 0; q < Q; q++) pop_out[g + q * V] = f[q];
            } else {
            float d = f[lex_q<Q>(0)], d_lo = 0.f;
#pragma unroll
            for (int i = 1; i < Q; i++) {
                if constexpr (EXACT_REST) {
                    float e;
                    two_sum(d, f[lex_q<Q>(i)], d, e);
                    d_lo += e;
                } else {
                    d += f[lex_q<Q>(i)];
                }
            }
            // Shan-Chen force from the psi ring (compile-time offsets); the
            // stencil is symmetric (w_a = w_-a, checked on the host), so each
            // pair +-e_a contributes w_a e_a (psi(x+e_a) - psi(x-e_a))
            float F[D];
#pragma unroll
            for (int c = 0; c < D; c++) F[c] = 0.f;
            auto psi_at = [&](int a) {
                const int em = D == 3 ? S::e(a, 2) : S::e(a, 1);
                const int ey = D == 3 ? S::e(a, 1) : 0;
                return sb[em + R][(D == 3 ? (R + ey) * HX : 0) + R + S::e(a, 0)];
            };
#pragma unroll
            for (int a = 0; a < S::QE; a++) {
                if (opposite_e<S>(a) < a) continue;
                const float dps = psi_at(a) - psi_at(opposite_e<S>(a));
#pragma unroll
                for (int c = 0; c < D; c++)
                    if (S::e(a, c) != 0) F[c] = fmaf(p.sw[a][c], dps, F[c]);
            }
            const float sc = neg_g * sb[R][(D == 3 ? R * HX : 0) + R];
#pragma unroll
            for (int c = 0; c < D; c++) F[c] *= sc;
            const float n = rho0 + d;
            float u[D];
            velocity<L, float>(f, n, F, u);
            // collision + push stream; rest population last, from mass conservation
            float u2 = 0.f, uF = 0.f;
#pragma unroll
            for (int c = 0; c < D; c++) {
                u2 = fmaf(u[c], u[c], u2);
                uF = fmaf(u[c], F[c], uF);
            }
            const float C0 = p.omega * d - p.om15 * n * u2 - p.fd * uF;
            const float a = p.om45 * n, b = p.om3 * n;
            float rest_pop = d, rest_lo = d_lo;
            float pend[Q];  // BGK: a direction's result computed with its opposite's
#pragma unroll
            for (int q = 1; q < Q; q++) {
                float out;
                if (MRT) {
                    collide_cell<L, S, true, float, false>(f, d, n, u, F, q, p, out);
                } else {
                    if (opposite_q<L>(q) > q) bgk_pair_fp32<L, S>(f, u, F, q, opposite_q<L>(q), p, C0, a, b, out,
                                                                  pend[opposite_q<L>(q)]);
                    else out = pend[q];
                }
                if constexpr (NOISE) out = __fadd_rn(out, nzs[(q - 1) * NT]);
                // __fsub_rn: no contraction with the product that made `out`
                // (at omega = 1 it is a plain multiply), so the rest population
                // balances exactly the rounded values that are stored
                if constexpr (EXACT_REST) {
                    float e;
                    two_sum(rest_pop, -out, rest_pop, e);
                    rest_lo += e;
                } else {
                    rest_pop = __fsub_rn(rest_pop, out);
                }
                int dst = X3[L::xi(q, 0) + 1] + Y3[L::xi(q, 1) + 1] + Z3[L::xi(q, D - 1) + 1];
                int qd = q;
                if constexpr (WALLS) {
                    if (fb[L::xi(q, D - 1) + 1][(D == 3 ? L::xi(q, 1) * HX : 0) + L::xi(q, 0)] == 0) {
                        dst = g;
                        qd = opposite_q<L>(q);
                    }
                }
                if constexpr (CS) __stcs(pop_out + (dst + qd * V), out);
                else pop_out[dst + qd * V] = out;
            }
            const float rest_out = EXACT_REST ? __fadd_rn(rest_pop, rest_lo) : rest_pop;
            if constexpr (CS) __stcs(pop_out + g, rest_out);
            else pop_out[g] = rest_out;
            }
        }
    }
}

// Resident CTAs per SM: BGK with paired halo loads four (64 registers, no
// spills), BGK with one halo cell per load three (80 registers, no spills; 5%
// faster than two at 256^3 D3Q19 E6, measured in one run), the dense MRT
// operator two.
// TILE (3D paired BGK only): index into kTiles; 0 keeps the default shape.
template <class L, class S, bool MRT, bool PAIRS = false, int TILE = 0>
__global__ void __launch_bounds__(TILE ? kTiles[TILE].tx * kTiles[TILE].ty : FusedShape<L, S>::NT,
                                  TILE ? kTiles[TILE].minb : (MRT ? 2 : (PAIRS ? 4 : 3)))
    k_fused(const float *__restrict__ pop, float *__restrict__ pop_out, const __grid_constant__ StepParams<L, S, float> p,
            const FusedGeom fg) {
    constexpr int TXT = TILE ? kTiles[TILE].tx : 0, TYT = TILE ? kTiles[TILE].ty : 0;
    constexpr bool MB = kTiles[TILE].mb != 0;
    using SH = FusedShape<L, S, TXT, TYT>;
    constexpr int D = L::D;
    extern __shared__ float smem[];
    const int Lm = D == 3 ? fg.L[2] : fg.L[1];
    bool dead = false;
    if constexpr (MB) {
        // initialised once here; each item re-initialises them (fused_tile)
        uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + SH::MB_RING * SH::HC);
        if (threadIdx.x == 0)
            for (int k = 0; k < SH::MB_RING; k++) mbar_init(&mbar[k], SH::NT);
        __syncthreads();
    }
    for (int item = blockIdx.x; item < fg.items; item += gridDim.x) {
        // order of the work items over the grid: 0 x fastest, then y, then
        // the chunk; 1 the chunk fastest (a tile column's chunks together);
        // 2 y fastest
        int ix, iy, ic;
        if (fg.order == 1) {
            ic = item % fg.chunks;
            const int r = item / fg.chunks;
            ix = r % fg.tiles_x;
            iy = D == 3 ? r / fg.tiles_x : 0;
        } else if (fg.order == 2 && D == 3) {
            iy = item % fg.tiles_y;
            const int r = item / fg.tiles_y;
            ix = r % fg.tiles_x;
            ic = r / fg.tiles_x;
        } else {
            ix = item % fg.tiles_x;
            const int rest = item / fg.tiles_x;
            iy = D == 3 ? rest % fg.tiles_y : 0;
            ic = D == 3 ? rest / fg.tiles_y : rest;
        }
        const int m0 = ic * fg.chunk;
        fused_tile<L, S, MRT, void, false, PAIRS, 0, TXT, TYT, false, kTiles[TILE].cs != 0, MB>(
            pop, pop_out, (int)fg.V, fg.L[0], fg.L[1], fg.L[2], ix * SH::TX, iy * SH::TY, m0, min(m0 + fg.chunk, Lm),
            p.neg_g, p.rho0, p, smem, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, fg.err,
            &dead);
    }
}

// Staged variants of the 3D paired single pass (STG_* flags, BGK): four CTAs
// per SM with one kind of staging (43 KB or 49 KB of shared memory each), two
// with both (83 KB).  Shared memory is aligned up to 128 bytes at run time
// (the TMA destinations), so the launch asks for 128 bytes more than the layout.
template <class L, class S, bool MRT, int STG>
__global__ void __launch_bounds__(FusedShape<L, S>::NT,
                                  ((STG & STG_OWN_TMA) && (STG & STG_HALO_ASYNC)) ? 2 : 4)
    k_fused_stg(const float *__restrict__ pop, float *__restrict__ pop_out,
                const __grid_constant__ StepParams<L, S, float> p, const FusedGeom fg,
                const __grid_constant__ CUtensorMap tmap) {
    using SH = FusedShape<L, S>;
    constexpr int D = L::D;
    extern __shared__ float smem_raw[];
    float *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u) / 4;
    uint64_t *bars =
        reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + SH::own_offset(STG) + 2 * SH::OWN_BOX_BYTES);
    if constexpr ((STG & STG_OWN_TMA) != 0) {
        if (threadIdx.x == 0) {
            mbar_init(&bars[0], 1);
            mbar_init(&bars[1], 1);
            mbar_fence_init();
        }
        __syncthreads();
    }
    unsigned k_issue = 0, k_wait = 0;
    bool dead = false;
    const int Lm = D == 3 ? fg.L[2] : fg.L[1];
    for (int item = blockIdx.x; item < fg.items; item += gridDim.x) {
        const int ix = item % fg.tiles_x;
        const int rest = item / fg.tiles_x;
        const int iy = rest % fg.tiles_y;
        const int ic = rest / fg.tiles_y;
        const int m0 = ic * fg.chunk;
        fused_tile<L, S, MRT, void, false, true, STG>(pop, pop_out, (int)fg.V, fg.L[0], fg.L[1], fg.L[2],
                                                      ix * SH::TX, iy * SH::TY, m0, min(m0 + fg.chunk, Lm), p.neg_g,
                                                      p.rho0, p, smem, nullptr, nullptr, nullptr, nullptr, &tmap,
                                                      bars, &k_issue, &k_wait, fg.err, &dead);
    }
}

// walls (BGK): the halo flags and walls' psi cost a few registers more, so two
// CTAs per SM
template <class L, class S>
__global__ void __launch_bounds__(FusedShape<L, S>::NT, 2)
    k_fused_walls(const float *__restrict__ pop, float *__restrict__ pop_out,
                  const __grid_constant__ StepParams<L, S, float> p, const FusedGeom fg,
                  const unsigned char *__restrict__ walls, const float *__restrict__ psi_w) {
    using SH = FusedShape<L, S>;
    constexpr int D = L::D;
    extern __shared__ float smem[];
    const int Lm = D == 3 ? fg.L[2] : fg.L[1];
    for (int item = blockIdx.x; item < fg.items; item += gridDim.x) {
        const int ix = item % fg.tiles_x;
        const int rest = item / fg.tiles_x;
        const int iy = D == 3 ? rest % fg.tiles_y : 0;
        const int ic = D == 3 ? rest / fg.tiles_y : rest;
        const int m0 = ic * fg.chunk;
        fused_tile<L, S, false, void, true>(pop, pop_out, (int)fg.V, fg.L[0], fg.L[1], fg.L[2], ix * SH::TX,
                                            iy * SH::TY, m0, min(m0 + fg.chunk, Lm), p.neg_g, p.rho0, p, smem,
                                            nullptr, nullptr, walls, psi_w);
    }
}

// CRNG: the generator (CRNG_*), a compile-time constant; ST its state type.
// Two CTAs per SM (128 registers, no spills): three (80 registers) spill and
// run no faster at 256^3 (MINSTD 1.318 / 1.327 ms, MMIX 1.465 / 1.472 ms)
template <class L, class S, int CRNG, bool PAIRS = false,
          class ST = typename std::conditional<CRNG == CRNG_MMIX, unsigned long long, unsigned int>::type>
__global__ void __launch_bounds__(FusedShape<L, S>::NT, 2)
    k_fused_noise(const float *__restrict__ pop, float *__restrict__ pop_out,
                  const __grid_constant__ StepParams<L, S, float> p, const FusedGeom fg, ST *__restrict__ seeds,
                  const __grid_constant__ NoiseParams<L, float> z) {
    using SH = FusedShape<L, S>;
    constexpr int D = L::D;
    extern __shared__ float smem[];
    const int Lm = D == 3 ? fg.L[2] : fg.L[1];
    for (int item = blockIdx.x; item < fg.items; item += gridDim.x) {
        const int ix = item % fg.tiles_x;
        const int rest = item / fg.tiles_x;
        const int iy = D == 3 ? rest % fg.tiles_y : 0;
        const int ic = D == 3 ? rest / fg.tiles_y : rest;
        const int m0 = ic * fg.chunk;
        fused_tile<L, S, false, ST, false, PAIRS, 0, 0, 0, false, false, false, CRNG>(
            pop, pop_out, (int)fg.V, fg.L[0], fg.L[1], fg.L[2], ix * SH::TX, iy * SH::TY, m0,
            min(m0 + fg.chunk, Lm), p.neg_g, p.rho0, p, smem, seeds, &z);
    }
}

// ---------------------------------------------------------------------------
// Batches of independent lattices (ragged sweeps): the lattices sit one after
// another in one SoA array (population q of cell g of lattice i at
// q*Vtot + base_i + g); every lattice has its own size, coupling G and FP32
// shift.  One launch steps every active lattice: CTAs take (lattice, tile,
// chunk) work items from an atomic queue, so lattices of any size share the
// GPU and retired lattices cost nothing.
// ---------------------------------------------------------------------------
struct BatchInst {
    int base, Lx, Ly, Lz;
    float neg_g, rho0;
    int active, pad;
};

// PAIRS: every lattice has an even Lx and an even first cell (base) and the
// total volume is even, so the paired halo loads of fused_tile stay aligned.
// Resident CTAs per SM as the single-lattice kernel's: four (BGK, paired
// loads, 64 registers) or three (BGK, one halo cell per load, 80 registers),
// no spills; two for the dense MRT operator.
// TXB (2D only): tile width, 0 for the single-lattice kernel's 256 cells;
// BATCH_TX_NARROW makes four times as many work items of a quarter the width
// (the same cells and arithmetic, so bit-identical), with the same registers
// per SM (twelve 64-thread CTAs for BGK)
constexpr int BATCH_TX_NARROW = 64;
constexpr int batch_min_blocks(bool mrt, bool pairs, int nt) { return (mrt ? 512 : (pairs ? 1024 : 768)) / nt; }
// ER: the compensated rest population (EXACT_REST of fused_tile); false only
// for 3D paired batches whose caller trades it for speed
template <class L, class S, bool MRT, bool PAIRS = false, int TXB = 0, bool ER = true>
__global__ void __launch_bounds__(FusedShape<L, S, TXB>::NT,
                                  batch_min_blocks(MRT, PAIRS, FusedShape<L, S, TXB>::NT))
    k_fused_batch(const float *__restrict__ pop, float *__restrict__ pop_out,
                  const __grid_constant__ StepParams<L, S, float> p, const BatchInst *__restrict__ inst,
                  const int4 *__restrict__ items, const int n_items, const int Vtot, int *counter, const int parity) {
    extern __shared__ float smem[];
    __shared__ int next;
    // launched as a programmatic dependent of the previous step: nothing is
    // read or written before that step has completed
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    // the other parity's queue is reset for the next step (not used by this one)
    if (blockIdx.x == 0 && threadIdx.x == 0) counter[parity ^ 1] = 0;
    while (true) {
        if (threadIdx.x == 0) next = atomicAdd(&counter[parity], 1);
        __syncthreads();
        const int it = next;
        __syncthreads();
        if (it >= n_items) {
            // no work left for this CTA: the next step may start placing its CTAs
            asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
            break;
        }
        const int4 w = items[it];  // lattice, x0, y0, m0 | m1 << 16
        const BatchInst I = inst[w.x];
        if (!I.active) continue;
        static_assert(TXB == 0 || L::D == 2, "narrow batch tiles: 2D");
        fused_tile<L, S, MRT, void, false, PAIRS, 0, TXB, 0, ER>(pop + I.base, pop_out + I.base, Vtot, I.Lx, I.Ly,
                                                                 I.Lz, w.y, w.z,
                                                  w.w & 0xffff, w.w >> 16, I.neg_g, I.rho0, p, smem);
    }
}

}  // namespace sclbm
