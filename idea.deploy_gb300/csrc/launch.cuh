// Type-erased launchers: one KernelOps table per (lattice, stencil, collision,
// precision).  Each lattice's instantiations live in their own translation unit
// (k_d2q9.cu, k_d3q19_e*.cu) so they compile in parallel.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <type_traits>

#include "batch.cuh"
#include "fused.cuh"
#include "kernels.cuh"
#include "noise.cuh"
#include "simple.cuh"

namespace sclbm {

// host-side description the launch parameters are filled from
struct HostSetup {
    int L[3];
    int64_t V;
    double rho0;
    double G;
    int psi_kind;
    const double *we;   // qe weights
    const double *A;    // q*q
    const double *B;    // q*K
    const double *Beq;  // q*K
    bool a_nonzero;
    double omega;       // BGK rate (factored single-pass collision), 0 if not BGK
    bool factored;      // FP64 BGK: the two-pass collision factored by opposite directions
    const double *w;    // q lattice weights
};

struct KernelOps {
    size_t step_size, eq_size;
    int kernels_per_step;
    void (*fill_step)(void *params, const HostSetup &h);
    void (*fill_eq)(void *params, const HostSetup &h);
    cudaError_t (*density)(const void *pop, void *dn, void *psi, const void *step_params, int grid,
                           cudaStream_t st);
    cudaError_t (*fcs)(const void *pop, void *pop_out, const void *dn, const void *psi,
                       const void *step_params, int grid, cudaStream_t st);
    cudaError_t (*velocity)(const void *pop, const void *dn, const void *psi, void *u,
                            const void *step_params, int grid, cudaStream_t st);
    // walls (flags 1 fluid / 0 wall, the walls' psi): density pass and fused step
    cudaError_t (*density_walls)(const void *pop, void *dn, void *psi, const unsigned char *walls, const void *psi_w,
                                 const void *step_params, int grid, cudaStream_t st);
    cudaError_t (*fcs_walls)(const void *pop, void *pop_out, const void *dn, const void *psi,
                             const unsigned char *walls, const void *step_params, int grid, cudaStream_t st);
    cudaError_t (*init_pop)(void *pop, const void *dn, const void *u, const void *eq_params, int grid,
                            cudaStream_t st);
    // occupancy-derived grid sizes (blocks) for a device with `sms` SMs
    void (*grids)(int sms, int *density_grid, int *fcs_grid);
    // single-pass step (FP32 only, else null): launcher, tile shape, resident CTAs per SM
    // tmap: host copy of the input buffer's CUtensorMap (used when fg.stg has STG_OWN_TMA)
    cudaError_t (*fused)(const void *pop, void *pop_out, const void *step_params, const FusedGeom &fg, int grid,
                         const void *tmap, cudaStream_t st);
    int fused_tx, fused_ty, fused_r;
    int (*fused_occupancy)(int pairs, int stg, int tile);  // of the paired-load instance when pairs != 0
    int fused_stg_mask;  // STG_* variants built for this kernel set (0: none)
    int fused_tile_mask; // kTiles shapes built (bit t) for the paired single pass (bit 0: the default)
    // batches of lattices (FP32 only, else null)
    // tx: tile width of a 2D batch (0: fused_tx; BATCH_TX_NARROW: the narrow tiles)
    // exact_rest 0 (3D paired BGK only): the rest population without the compensated sums
    cudaError_t (*batch_step)(const void *pop, void *pop_out, const void *sp, const BatchInst *inst, const int4 *items,
                              int n_items, int Vtot, int *counter, int parity, int pairs, int tx, int exact_rest,
                              int grid, cudaStream_t st);
    int (*batch_occupancy)(int pairs, int tx);  // resident CTAs per SM of the batch kernel
    cudaError_t (*batch_density)(const void *pop, void *dn, void *psi, const void *sp, const BatchInst *inst, int n_inst,
                                 int Vtot, int gx, cudaStream_t st);
    cudaError_t (*batch_moments)(const void *pop, const void *dn, const void *psi, void *u_old, const void *sp,
                                 const BatchInst *inst, int n_inst, int Vtot, double *partials, int gx, cudaStream_t st);
    // exact per-lattice mass, rest-population correction, centre/last-cell density
    cudaError_t (*batch_mass)(const void *pop, const BatchInst *inst, int n_inst, int Vtot, double *partials, int gx,
                              cudaStream_t st);
    cudaError_t (*batch_add_rest)(void *pop, const BatchInst *inst, int n_inst, int Vtot, const float *delta, int gx,
                                  cudaStream_t st);
    cudaError_t (*batch_probe)(const void *pop, const BatchInst *inst, int n_inst, int Vtot, double *out, int rad,
                               cudaStream_t st);
    // fluctuating step (BGK only, else null): parameter block, its filler from the
    // noise operator (m2var[nr], coef[q*nr]) and the launcher; grid from occupancy
    size_t noise_size;
    void (*fill_noise)(void *params, int kind, int indep, const double *m2var, const double *coef);
    cudaError_t (*fcs_noise)(const void *pop, void *pop_out, const void *dn, const void *psi, void *seeds,
                             const void *step_params, const void *noise_params, int grid, cudaStream_t st);
    int (*noise_occupancy)();
    // single-pass fluctuating step (FP32 BGK only, else null)
    cudaError_t (*fused_noise)(const void *pop, void *pop_out, const void *step_params, const FusedGeom &fg,
                               void *seeds, const void *noise_params, int grid, cudaStream_t st);
    int (*fused_noise_occupancy)(int kind);  // kind: CRNG_*
    unsigned (*noise_mask)(int q);  // nonzero pattern the single-pass noise kernel assumes
    // single-pass step with walls (FP32 BGK only, else null)
    cudaError_t (*fused_walls)(const void *pop, void *pop_out, const void *step_params, const FusedGeom &fg,
                               const unsigned char *walls, const void *psi_w, int grid, cudaStream_t st);
    int (*fused_walls_occupancy)();
    // the "simple" step family (FP64 only, else null)
    cudaError_t (*simple_inlet)(void *pop, void *dn, void *u, const unsigned char *walls, const SimpleParams &p,
                                int grid, cudaStream_t st);
    cudaError_t (*simple_outlet)(void *pop, void *dn, void *u, const unsigned char *walls, const SimpleParams &p,
                                 int grid, cudaStream_t st);
    cudaError_t (*simple_moments)(const void *pop, void *dn, void *u, void *psi, const unsigned char *walls,
                                  const SimpleParams &p, int grid, cudaStream_t st);
    cudaError_t (*simple_collide)(int sc, int push, const void *pop, void *pop_out, const void *dn, void *u,
                                  const void *psi, const unsigned char *walls, const SimpleParams &p, int grid,
                                  cudaStream_t st);
    cudaError_t (*simple_stream)(const void *pop, void *pop_out, const unsigned char *walls, const SimpleParams &p,
                                 int grid, cudaStream_t st);
};

template <class L, class S, bool MRT, class Real, bool STRICT>
struct Ops {
    using SP = StepParams<L, S, Real>;
    using EP = EqParams<L, Real>;
    static constexpr int D = L::D, Q = L::Q, K = Mono<L::D>::K;

    static void fill_geo(Geometry<Real> &g, const HostSetup &h) {
        for (int d = 0; d < 3; d++) g.L[d] = h.L[d];
        g.V = h.V;
    }
    static void fill_step(void *params, const HostSetup &h) {
        SP *p = static_cast<SP *>(params);
        std::memset(p, 0, sizeof(SP));
        fill_geo(p->geo, h);
        p->rho0 = (Real)h.rho0;
        p->neg_g = (Real)(-h.G);
        p->psi_kind = h.psi_kind;
        p->a_nonzero = h.a_nonzero ? 1 : 0;
        p->factored = h.factored ? 1 : 0;
        for (int a = 0; a < S::QE; a++)
            for (int d = 0; d < D; d++)
                p->sw[a][d] = (Real)((double)S::e(a, d) * h.we[a]);
        for (int i = 0; i < Q; i++)
            for (int j = 0; j < Q; j++) p->A[i][j] = (Real)h.A[i * Q + j];
        for (int i = 0; i < Q; i++)
            for (int k = 0; k < K; k++) p->B[i][k] = (Real)h.B[i * K + k];
        const double w = h.omega;
        p->omega = (Real)w;
        p->om15 = (Real)(1.5 * w);
        p->om3 = (Real)(3.0 * w);
        p->om45 = (Real)(4.5 * w);
        p->fc = (Real)(9.0 * (1.0 - 0.5 * w));
        p->fd = (Real)(3.0 * (1.0 - 0.5 * w));
        for (int i = 0; i < Q; i++) p->wq[i] = (Real)(h.w ? h.w[i] : 0.0);
    }
    static void fill_eq(void *params, const HostSetup &h) {
        EP *p = static_cast<EP *>(params);
        std::memset(p, 0, sizeof(EP));
        fill_geo(p->geo, h);
        p->rho0 = (Real)h.rho0;
        for (int i = 0; i < Q; i++)
            for (int k = 0; k < K; k++) p->B[i][k] = (Real)h.Beq[i * K + k];
    }
    static cudaError_t density(const void *pop, void *dn, void *psi, const void *sp, int grid, cudaStream_t st) {
        const SP *p = static_cast<const SP *>(sp);
        k_density_psi<L, Real><<<grid, 256, 0, st>>>((const Real *)pop, (Real *)dn, (Real *)psi, p->geo, p->rho0,
                                                     p->psi_kind);
        return cudaGetLastError();
    }
    static cudaError_t fcs(const void *pop, void *pop_out, const void *dn, const void *psi, const void *sp, int grid,
                           cudaStream_t st) {
        k_fcs<L, S, MRT, Real, STRICT><<<grid, 128, 0, st>>>((const Real *)pop, (Real *)pop_out, (const Real *)dn,
                                                     (const Real *)psi, *static_cast<const SP *>(sp));
        return cudaGetLastError();
    }
    static cudaError_t velocity(const void *pop, const void *dn, const void *psi, void *u, const void *sp, int grid,
                                cudaStream_t st) {
        k_velocity<L, S, Real, STRICT><<<grid, 128, 0, st>>>((const Real *)pop, (const Real *)dn, (const Real *)psi,
                                                          (Real *)u, *static_cast<const SP *>(sp));
        return cudaGetLastError();
    }
    static cudaError_t density_walls(const void *pop, void *dn, void *psi, const unsigned char *walls,
                                     const void *psi_w, const void *sp, int grid, cudaStream_t st) {
        const SP *p = static_cast<const SP *>(sp);
        k_density_psi_walls<L, Real><<<grid, 256, 0, st>>>((const Real *)pop, (Real *)dn, (Real *)psi, walls,
                                                           (const Real *)psi_w, p->geo, p->rho0, p->psi_kind);
        return cudaGetLastError();
    }
    static cudaError_t fcs_walls(const void *pop, void *pop_out, const void *dn, const void *psi,
                                 const unsigned char *walls, const void *sp, int grid, cudaStream_t st) {
        k_fcs_walls<L, S, MRT, Real, STRICT><<<grid, 128, 0, st>>>((const Real *)pop, (Real *)pop_out,
                                                                   (const Real *)dn, (const Real *)psi, walls,
                                                                   *static_cast<const SP *>(sp));
        return cudaGetLastError();
    }
    static cudaError_t init_pop(void *pop, const void *dn, const void *u, const void *ep, int grid, cudaStream_t st) {
        k_init_pop<L, Real, STRICT><<<grid, 128, 0, st>>>((Real *)pop, (const Real *)dn, (const Real *)u,
                                                  *static_cast<const EP *>(ep));
        return cudaGetLastError();
    }
    static void grids(int sms, int *dg, int *fg) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_density_psi<L, Real>, 256, 0);
        *dg = sms * (b > 0 ? b : 1);
        b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fcs<L, S, MRT, Real, STRICT>, 128, 0);
        *fg = sms * (b > 0 ? b : 1);
    }
    // staged variants: 3D, even radius, BGK, FP32
    static constexpr bool STG_BUILT = std::is_same<Real, float>::value && L::D == 3 && S::R % 2 == 0 && !MRT;
    static constexpr int STG_MASK = STG_BUILT ? 3 : 0;
    static constexpr int TILE_MASK = STG_BUILT ? (1 << N_TILES) - 1 : 1;
    template <int TILE>
    static constexpr int tile_smem() {
        using SH = FusedShape<L, S, kTiles[TILE].tx, kTiles[TILE].ty>;
        return kTiles[TILE].mb ? SH::MB_SMEM : SH::SMEM;
    }
    template <int TILE>
    static void allow_tile_smem() {
        static bool done[64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= 64 || !done[dev]) {
            cudaFuncSetAttribute(k_fused<L, S, MRT, true, TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tile_smem<TILE>());
            if (dev >= 0 && dev < 64) done[dev] = true;
        }
    }
    template <int TILE>
    static cudaError_t launch_tile(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg, int grid,
                                   cudaStream_t st) {
        using SH = FusedShape<L, S, kTiles[TILE].tx, kTiles[TILE].ty>;
        allow_tile_smem<TILE>();
        k_fused<L, S, MRT, true, TILE><<<grid, SH::NT, tile_smem<TILE>(), st>>>(
            (const float *)pop, (float *)pop_out, *static_cast<const SP *>(sp), fg);
        return cudaGetLastError();
    }
    template <int TILE>
    static int occupancy_tile() {
        using SH = FusedShape<L, S, kTiles[TILE].tx, kTiles[TILE].ty>;
        allow_tile_smem<TILE>();
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused<L, S, MRT, true, TILE>, SH::NT, tile_smem<TILE>());
        return b > 0 ? b : 1;
    }
    template <int STG>
    static cudaError_t launch_stg(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg, int grid,
                                  const void *tmap, cudaStream_t st) {
        using SH = FusedShape<L, S>;
        static bool done[64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= 64 || !done[dev]) {
            cudaFuncSetAttribute(k_fused_stg<L, S, MRT, STG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 SH::stg_smem(STG) + 128);
            if (dev >= 0 && dev < 64) done[dev] = true;
        }
        if (!tmap && (STG & STG_OWN_TMA)) return cudaErrorInvalidValue;
        CUtensorMap none;
        std::memset(&none, 0, sizeof(none));
        k_fused_stg<L, S, MRT, STG><<<grid, SH::NT, SH::stg_smem(STG) + 128, st>>>(
            (const float *)pop, (float *)pop_out, *static_cast<const SP *>(sp), fg,
            tmap ? *static_cast<const CUtensorMap *>(tmap) : none);
        return cudaGetLastError();
    }
    static cudaError_t fused(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg, int grid,
                             const void *tmap, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            using SH = FusedShape<L, S>;
            allow_smem();
            if constexpr (STG_BUILT) {
                if (fg.pairs && fg.stg == 1) return launch_stg<1>(pop, pop_out, sp, fg, grid, tmap, st);
                if (fg.pairs && fg.stg == 2) return launch_stg<2>(pop, pop_out, sp, fg, grid, tmap, st);
                if (fg.pairs && fg.stg == 3) return launch_stg<3>(pop, pop_out, sp, fg, grid, tmap, st);
                if (fg.pairs && !fg.stg && fg.tile == 1) return launch_tile<1>(pop, pop_out, sp, fg, grid, st);
                if (fg.pairs && !fg.stg && fg.tile == 2) return launch_tile<2>(pop, pop_out, sp, fg, grid, st);
                if (fg.pairs && !fg.stg && fg.tile == 3) return launch_tile<3>(pop, pop_out, sp, fg, grid, st);
                if (fg.pairs && !fg.stg && fg.tile == 4) return launch_tile<4>(pop, pop_out, sp, fg, grid, st);
                if (fg.pairs && !fg.stg && fg.tile == 5) return launch_tile<5>(pop, pop_out, sp, fg, grid, st);
            }
            if (fg.stg || fg.tile) return cudaErrorNotSupported;
            if constexpr (L::D == 3 && S::R % 2 == 0) {
                if (fg.pairs) {
                    k_fused<L, S, MRT, true><<<grid, SH::NT, SH::SMEM, st>>>((const float *)pop, (float *)pop_out,
                                                                             *static_cast<const SP *>(sp), fg);
                    return cudaGetLastError();
                }
            }
            k_fused<L, S, MRT><<<grid, SH::NT, SH::SMEM, st>>>((const float *)pop, (float *)pop_out,
                                                               *static_cast<const SP *>(sp), fg);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    // the single-pass kernel's shared memory (psi ring + stage) exceeds the 48 KB default
    static void allow_smem() {
        if constexpr (std::is_same<Real, float>::value) {
            static bool done[64] = {};  // per device
            int dev = 0;
            cudaGetDevice(&dev);
            if (dev < 0 || dev >= 64 || !done[dev]) {
                cudaFuncSetAttribute(k_fused<L, S, MRT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     FusedShape<L, S>::SMEM);
                if constexpr (L::D == 3 && S::R % 2 == 0)
                    cudaFuncSetAttribute(k_fused<L, S, MRT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         FusedShape<L, S>::SMEM);
                if (dev >= 0 && dev < 64) done[dev] = true;
            }
        }
    }
    template <int STG>
    static int occupancy_stg() {
        using SH = FusedShape<L, S>;
        cudaFuncSetAttribute(k_fused_stg<L, S, MRT, STG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SH::stg_smem(STG) + 128);
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused_stg<L, S, MRT, STG>, SH::NT, SH::stg_smem(STG) + 128);
        return b > 0 ? b : 1;
    }
    static int fused_occupancy(int pairs, int stg, int tile) {
        if constexpr (std::is_same<Real, float>::value) {
            using SH = FusedShape<L, S>;
            allow_smem();
            if constexpr (STG_BUILT) {
                if (pairs && stg == 1) return occupancy_stg<1>();
                if (pairs && stg == 2) return occupancy_stg<2>();
                if (pairs && stg == 3) return occupancy_stg<3>();
                if (pairs && tile == 1) return occupancy_tile<1>();
                if (pairs && tile == 2) return occupancy_tile<2>();
                if (pairs && tile == 3) return occupancy_tile<3>();
                if (pairs && tile == 4) return occupancy_tile<4>();
                if (pairs && tile == 5) return occupancy_tile<5>();
            }
            int b = 0;
            if constexpr (L::D == 3 && S::R % 2 == 0) {
                if (pairs) {
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused<L, S, MRT, true>, SH::NT, SH::SMEM);
                    return b > 0 ? b : 1;
                }
            }
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused<L, S, MRT>, SH::NT, SH::SMEM);
            return b > 0 ? b : 1;
        }
        return 0;
    }
    template <bool PAIRS, int TXB, bool ER = true>
    static void batch_allow_smem() {
        using SH = FusedShape<L, S, TXB>;
        static bool done[64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= 64 || !done[dev]) {
            cudaFuncSetAttribute(k_fused_batch<L, S, MRT, PAIRS, TXB, ER>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SH::SMEM);
            if (dev >= 0 && dev < 64) done[dev] = true;
        }
    }
    template <bool PAIRS, int TXB, bool ER = true>
    static cudaError_t batch_launch(const void *pop, void *pop_out, const void *sp, const BatchInst *inst,
                                    const int4 *items, int n_items, int Vtot, int *counter, int parity, int grid,
                                    cudaStream_t st) {
        using SH = FusedShape<L, S, TXB>;
        batch_allow_smem<PAIRS, TXB, ER>();
        // programmatic dependent launch: a step's CTAs are placed while the
        // previous step's last items finish, and wait (griddepcontrol.wait)
        // for its completion before they read anything
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(SH::NT);
        cfg.dynamicSmemBytes = SH::SMEM;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_fused_batch<L, S, MRT, PAIRS, TXB, ER>, (const float *)pop, (float *)pop_out,
                                  *static_cast<const SP *>(sp), inst, items, n_items, Vtot, counter, parity);
    }
    static cudaError_t batch_step(const void *pop, void *pop_out, const void *sp, const BatchInst *inst,
                                  const int4 *items, int n_items, int Vtot, int *counter, int parity, int pairs,
                                  int tx, int exact_rest, int grid, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            if constexpr (L::D == 3 && S::R % 2 == 0 && !MRT) {
                if (pairs && !exact_rest)
                    return batch_launch<true, 0, false>(pop, pop_out, sp, inst, items, n_items, Vtot, counter, parity,
                                                        grid, st);
            }
            if (!exact_rest) return cudaErrorNotSupported;
            if constexpr (L::D == 3 && S::R % 2 == 0) {
                if (pairs)
                    return batch_launch<true, 0>(pop, pop_out, sp, inst, items, n_items, Vtot, counter, parity, grid,
                                                 st);
            }
            if constexpr (L::D == 2) {
                if (tx == BATCH_TX_NARROW)
                    return batch_launch<false, BATCH_TX_NARROW>(pop, pop_out, sp, inst, items, n_items, Vtot, counter,
                                                                parity, grid, st);
            }
            if (tx != 0 && tx != FusedShape<L, S>::TX) return cudaErrorInvalidValue;
            return batch_launch<false, 0>(pop, pop_out, sp, inst, items, n_items, Vtot, counter, parity, grid, st);
        }
        return cudaErrorNotSupported;
    }
    template <bool PAIRS, int TXB>
    static int batch_occ() {
        using SH = FusedShape<L, S, TXB>;
        int b = 0;
        batch_allow_smem<PAIRS, TXB>();
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused_batch<L, S, MRT, PAIRS, TXB>, SH::NT, SH::SMEM);
        return b > 0 ? b : 1;
    }
    static int batch_occupancy(int pairs, int tx) {
        if constexpr (std::is_same<Real, float>::value) {
            if constexpr (L::D == 3 && S::R % 2 == 0) {
                if (pairs) return batch_occ<true, 0>();
            }
            if constexpr (L::D == 2) {
                if (tx == BATCH_TX_NARROW) return batch_occ<false, BATCH_TX_NARROW>();
            }
            return batch_occ<false, 0>();
        }
        return 1;
    }
    static cudaError_t batch_density(const void *pop, void *dn, void *psi, const void *sp, const BatchInst *inst,
                                     int n_inst, int Vtot, int gx, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            k_batch_density<L><<<dim3(gx, n_inst), BATCH_THREADS, 0, st>>>(
                (const float *)pop, (float *)dn, (float *)psi, inst, Vtot, static_cast<const SP *>(sp)->psi_kind);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    static cudaError_t batch_moments(const void *pop, const void *dn, const void *psi, void *u_old, const void *sp,
                                     const BatchInst *inst, int n_inst, int Vtot, double *partials, int gx,
                                     cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            k_batch_moments<L, S><<<dim3(gx, n_inst), BATCH_THREADS, 0, st>>>(
                (const float *)pop, (const float *)dn, (const float *)psi, (float *)u_old, *static_cast<const SP *>(sp),
                inst, Vtot, partials);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    static cudaError_t batch_mass(const void *pop, const BatchInst *inst, int n_inst, int Vtot, double *partials,
                                  int gx, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            k_batch_mass<L><<<dim3(gx, n_inst), BATCH_THREADS, 0, st>>>((const float *)pop, inst, Vtot, partials);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    static cudaError_t batch_add_rest(void *pop, const BatchInst *inst, int n_inst, int Vtot, const float *delta,
                                      int gx, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            k_batch_add_rest<L><<<dim3(gx, n_inst), BATCH_THREADS, 0, st>>>((float *)pop, inst, Vtot, delta);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    static cudaError_t batch_probe(const void *pop, const BatchInst *inst, int n_inst, int Vtot, double *out, int rad,
                                   cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value) {
            k_batch_probe<L><<<n_inst, 32, 0, st>>>((const float *)pop, inst, Vtot, out, rad);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    using NP = NoiseParams<L, Real>;
    static void fill_noise(void *params, int kind, int indep, const double *m2var, const double *coef) {
        NP *z = static_cast<NP *>(params);
        std::memset(z, 0, sizeof(NP));
        z->kind = kind;
        z->indep = indep;
        for (int k = 0; k < NP::NR; k++) z->m2var[k] = (Real)m2var[k];
        for (int q = 0; q < Q; q++)
            for (int k = 0; k < NP::NR; k++) z->coef[q][k] = (Real)coef[q * NP::NR + k];
    }
    static cudaError_t fcs_noise(const void *pop, void *pop_out, const void *dn, const void *psi, void *seeds,
                                 const void *sp, const void *np, int grid, cudaStream_t st) {
        if constexpr (!MRT) {
            const NP &z = *static_cast<const NP *>(np);
            if (z.kind == CRNG_MMIX)
                k_fcs_noise<L, S, Real, STRICT, unsigned long long><<<grid, 128, 0, st>>>(
                    (const Real *)pop, (Real *)pop_out, (const Real *)dn, (const Real *)psi,
                    (unsigned long long *)seeds, *static_cast<const SP *>(sp), z);
            else
                k_fcs_noise<L, S, Real, STRICT, unsigned int><<<grid, 128, 0, st>>>(
                    (const Real *)pop, (Real *)pop_out, (const Real *)dn, (const Real *)psi, (unsigned int *)seeds,
                    *static_cast<const SP *>(sp), z);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    template <int CRNG, bool PAIRS>
    static cudaError_t launch_noise(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg, void *seeds,
                                    const NP &z, int grid, cudaStream_t st) {
        using SH = FusedShape<L, S>;
        using ST = typename std::conditional<CRNG == CRNG_MMIX, unsigned long long, unsigned int>::type;
        k_fused_noise<L, S, CRNG, PAIRS><<<grid, SH::NT, SH::NSMEM, st>>>(
            (const float *)pop, (float *)pop_out, *static_cast<const SP *>(sp), fg, (ST *)seeds, z);
        return cudaGetLastError();
    }
    template <bool PAIRS>
    static cudaError_t launch_noise_kind(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg,
                                         void *seeds, const NP &z, int grid, cudaStream_t st) {
        switch (z.kind) {
        case CRNG_MINSTD: return launch_noise<CRNG_MINSTD, PAIRS>(pop, pop_out, sp, fg, seeds, z, grid, st);
        case CRNG_NUMREC: return launch_noise<CRNG_NUMREC, PAIRS>(pop, pop_out, sp, fg, seeds, z, grid, st);
        case CRNG_MMIX: return launch_noise<CRNG_MMIX, PAIRS>(pop, pop_out, sp, fg, seeds, z, grid, st);
        default: return cudaErrorInvalidValue;
        }
    }
    static cudaError_t fused_noise(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg, void *seeds,
                                   const void *np, int grid, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value && !MRT) {
            allow_smem_noise();
            const NP &z = *static_cast<const NP *>(np);
            if constexpr (L::D == 3 && S::R % 2 == 0) {
                if (fg.pairs) return launch_noise_kind<true>(pop, pop_out, sp, fg, seeds, z, grid, st);
            }
            return launch_noise_kind<false>(pop, pop_out, sp, fg, seeds, z, grid, st);
        }
        return cudaErrorNotSupported;
    }
    template <bool PAIRS>
    static void allow_smem_noise_pairs() {
        constexpr int n = FusedShape<L, S>::NSMEM;
        cudaFuncSetAttribute(k_fused_noise<L, S, CRNG_MINSTD, PAIRS>, cudaFuncAttributeMaxDynamicSharedMemorySize, n);
        cudaFuncSetAttribute(k_fused_noise<L, S, CRNG_NUMREC, PAIRS>, cudaFuncAttributeMaxDynamicSharedMemorySize, n);
        cudaFuncSetAttribute(k_fused_noise<L, S, CRNG_MMIX, PAIRS>, cudaFuncAttributeMaxDynamicSharedMemorySize, n);
    }
    static void allow_smem_noise() {
        if constexpr (std::is_same<Real, float>::value && !MRT) {
            static bool done[64] = {};  // per device
            int dev = 0;
            cudaGetDevice(&dev);
            if (dev < 0 || dev >= 64 || !done[dev]) {
                allow_smem_noise_pairs<false>();
                if constexpr (L::D == 3 && S::R % 2 == 0) allow_smem_noise_pairs<true>();
                if (dev >= 0 && dev < 64) done[dev] = true;
            }
        }
    }
    static int fused_noise_occupancy(int kind) {
        int b = 0;
        if constexpr (std::is_same<Real, float>::value && !MRT) {
            using SH = FusedShape<L, S>;
            allow_smem_noise();
            if (kind == CRNG_MINSTD)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused_noise<L, S, CRNG_MINSTD>, SH::NT, SH::NSMEM);
            else if (kind == CRNG_NUMREC)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused_noise<L, S, CRNG_NUMREC>, SH::NT, SH::NSMEM);
            else
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused_noise<L, S, CRNG_MMIX>, SH::NT, SH::NSMEM);
        }
        return b > 0 ? b : 1;
    }
    static int noise_occupancy() {
        int b = 0;
        if constexpr (!MRT)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fcs_noise<L, S, Real, STRICT, unsigned long long>, 128,
                                                          0);
        return b > 0 ? b : 1;
    }
    static constexpr bool F64 = std::is_same<Real, double>::value;
    static void allow_smem_walls() {
        if constexpr (std::is_same<Real, float>::value && !MRT) {
            static bool done[64] = {};  // per device
            int dev = 0;
            cudaGetDevice(&dev);
            if (dev < 0 || dev >= 64 || !done[dev]) {
                cudaFuncSetAttribute(k_fused_walls<L, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     FusedShape<L, S>::WSMEM);
                if (dev >= 0 && dev < 64) done[dev] = true;
            }
        }
    }
    static cudaError_t fused_walls(const void *pop, void *pop_out, const void *sp, const FusedGeom &fg,
                                   const unsigned char *walls, const void *psi_w, int grid, cudaStream_t st) {
        if constexpr (std::is_same<Real, float>::value && !MRT) {
            using SH = FusedShape<L, S>;
            allow_smem_walls();
            k_fused_walls<L, S><<<grid, SH::NT, SH::WSMEM, st>>>((const float *)pop, (float *)pop_out,
                                                                 *static_cast<const SP *>(sp), fg, walls,
                                                                 (const float *)psi_w);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    static int fused_walls_occupancy() {
        int b = 0;
        if constexpr (std::is_same<Real, float>::value && !MRT) {
            using SH = FusedShape<L, S>;
            allow_smem_walls();
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused_walls<L, S>, SH::NT, SH::WSMEM);
        }
        return b > 0 ? b : 1;
    }
    static cudaError_t simple_inlet(void *pop, void *dn, void *u, const unsigned char *walls, const SimpleParams &sp,
                                    int grid, cudaStream_t st) {
        if constexpr (F64)
            k_simple_inlet<L, STRICT><<<grid, 256, 0, st>>>((double *)pop, (double *)dn, (double *)u, walls, sp);
        else
            k_simple_inlet_f32<L><<<grid, 256, 0, st>>>((float *)pop, (float *)dn, (float *)u, walls, sp);
        return cudaGetLastError();
    }
    static cudaError_t simple_outlet(void *pop, void *dn, void *u, const unsigned char *walls, const SimpleParams &sp,
                                     int grid, cudaStream_t st) {
        k_simple_outlet<L, Real><<<grid, 256, 0, st>>>((Real *)pop, (Real *)dn, (Real *)u, walls, sp);
        return cudaGetLastError();
    }
    static cudaError_t simple_moments(const void *pop, void *dn, void *u, void *psi, const unsigned char *walls,
                                      const SimpleParams &sp, int grid, cudaStream_t st) {
        if constexpr (F64)
            k_simple_moments<L, STRICT><<<grid, 256, 0, st>>>((const double *)pop, (double *)dn, (double *)u,
                                                              (double *)psi, walls, sp);
        else
            k_simple_moments_f32<L><<<grid, 256, 0, st>>>((const float *)pop, (float *)dn, (float *)u, (float *)psi,
                                                          walls, sp);
        return cudaGetLastError();
    }
    static cudaError_t simple_collide(int sc, int push, const void *pop, void *pop_out, const void *dn, void *u,
                                      const void *psi, const unsigned char *walls, const SimpleParams &sp, int grid,
                                      cudaStream_t st) {
        const Real *a = (const Real *)pop, *n = (const Real *)dn, *ps = (const Real *)psi;
        Real *b = (Real *)pop_out, *uu = (Real *)u;
        if constexpr (F64) {
            if (!sc)
                k_simple_collide<L, S, STRICT, false, true><<<grid, 128, 0, st>>>(a, b, n, uu, ps, walls, sp);
            else if (push)
                k_simple_collide<L, S, STRICT, true, true><<<grid, 128, 0, st>>>(a, b, n, uu, ps, walls, sp);
            else
                k_simple_collide<L, S, STRICT, true, false><<<grid, 128, 0, st>>>(a, b, n, uu, ps, walls, sp);
        } else {
            if (!sc)
                k_simple_collide_f32<L, S, false, true><<<grid, 128, 0, st>>>(a, b, n, uu, ps, walls, sp);
            else if (push)
                k_simple_collide_f32<L, S, true, true><<<grid, 128, 0, st>>>(a, b, n, uu, ps, walls, sp);
            else
                k_simple_collide_f32<L, S, true, false><<<grid, 128, 0, st>>>(a, b, n, uu, ps, walls, sp);
        }
        return cudaGetLastError();
    }
    static cudaError_t simple_stream(const void *pop, void *pop_out, const unsigned char *walls, const SimpleParams &sp,
                                     int grid, cudaStream_t st) {
        k_simple_stream<L, Real><<<grid, 128, 0, st>>>((const Real *)pop, (Real *)pop_out, walls, sp);
        return cudaGetLastError();
    }
    static const KernelOps *ops() {
        constexpr bool f32 = std::is_same<Real, float>::value;
        using SH = FusedShape<L, S>;
        static const KernelOps o = {sizeof(SP), sizeof(EP), f32 ? 1 : 2, &fill_step, &fill_eq, &density,
                                    &fcs, &velocity, &density_walls, &fcs_walls, &init_pop, &grids,
                                    f32 ? &fused : nullptr, SH::TX, SH::TY, SH::R,
                                    f32 ? &fused_occupancy : nullptr, STG_MASK, TILE_MASK,
                                    f32 ? &batch_step : nullptr, &batch_occupancy, f32 ? &batch_density : nullptr,
                                    f32 ? &batch_moments : nullptr, f32 ? &batch_mass : nullptr,
                                    f32 ? &batch_add_rest : nullptr, f32 ? &batch_probe : nullptr,
                                    sizeof(NP), MRT ? nullptr : &fill_noise, MRT ? nullptr : &fcs_noise,
                                    &noise_occupancy, (f32 && !MRT) ? &fused_noise : nullptr,
                                    &fused_noise_occupancy, &NoiseMask<L>::m,
                                    (f32 && !MRT) ? &fused_walls : nullptr, &fused_walls_occupancy,
                                    &simple_inlet, &simple_outlet, &simple_moments, &simple_collide,
                                    &simple_stream};
        return &o;
    }
};

// One translation unit per (lattice, stencil, precision/arithmetic) so that
// the instantiations compile in parallel; each defines ops_<lat>_e<order>_<v>
// (v: f32 = FP32-shifted, f64 = FP64 fused arithmetic, f64s = FP64 reference
// arithmetic, i.e. the reference's evaluation order without FMA).
#define SCLBM_OPS_TU(NAME, L, S, REAL, STRICT)                                                    \
    const KernelOps *NAME(bool mrt) {                                                             \
        return mrt ? Ops<L, S, true, REAL, STRICT>::ops() : Ops<L, S, false, REAL, STRICT>::ops(); \
    }

#define SCLBM_DECLARE_OPS(LAT)                                                                    \
    const KernelOps *ops_##LAT##_e4_f32(bool);                                                    \
    const KernelOps *ops_##LAT##_e4_f64(bool);                                                    \
    const KernelOps *ops_##LAT##_e4_f64s(bool);                                                   \
    const KernelOps *ops_##LAT##_e6_f32(bool);                                                    \
    const KernelOps *ops_##LAT##_e6_f64(bool);                                                    \
    const KernelOps *ops_##LAT##_e6_f64s(bool);                                                   \
    const KernelOps *ops_##LAT##_e8_f32(bool);                                                    \
    const KernelOps *ops_##LAT##_e8_f64(bool);                                                    \
    const KernelOps *ops_##LAT##_e8_f64s(bool);
SCLBM_DECLARE_OPS(d2q9)
SCLBM_DECLARE_OPS(d3q19)

// kernel set for (dimension, stencil order, collision, precision, arithmetic)
inline const KernelOps *select_ops(int dim, int order, bool mrt, bool fp32, bool strict) {
    using Fn = const KernelOps *(*)(bool);
    static const Fn t2[3][3] = {{ops_d2q9_e4_f32, ops_d2q9_e4_f64, ops_d2q9_e4_f64s},
                                {ops_d2q9_e6_f32, ops_d2q9_e6_f64, ops_d2q9_e6_f64s},
                                {ops_d2q9_e8_f32, ops_d2q9_e8_f64, ops_d2q9_e8_f64s}};
    static const Fn t3[3][3] = {{ops_d3q19_e4_f32, ops_d3q19_e4_f64, ops_d3q19_e4_f64s},
                                {ops_d3q19_e6_f32, ops_d3q19_e6_f64, ops_d3q19_e6_f64s},
                                {ops_d3q19_e8_f32, ops_d3q19_e8_f64, ops_d3q19_e8_f64s}};
    const int o = order == 4 ? 0 : order == 6 ? 1 : order == 8 ? 2 : -1;
    if (o < 0 || (dim != 2 && dim != 3)) return nullptr;
    const int v = fp32 ? 0 : strict ? 2 : 1;
    return (dim == 2 ? t2 : t3)[o][v](mrt);
}

}  // namespace sclbm
