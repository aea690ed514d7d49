/*
 * sclbm.h -- C ABI of the GB300-native Shan-Chen multiphase LBM time step.
 *
 * One handle = one periodic lattice resident in HBM (populations stored SoA,
 * q-major, x fastest), stepped by hand-written sm_103a kernels.  Every call
 * returns an int status (SCLBM_OK == 0) and never aborts; host buffers are
 * owned by the caller, device state by the handle.  Calls on one handle are
 * not thread-safe; distinct handles are independent.
 *
 * The entry points replace the generated kernels and the per-step dispatch of
 * the reference (lullimat/idea.deploy, package idpy):
 *
 *   sclbm_create            ShanChenMultiPhase.__init__ / SetupRoot / InitVars /
 *                           InitMemory          idpy/LBM/MultiPhase.py:141-155,1941-2169
 *   sclbm_set_density/_velocity
 *                           sims_idpy_memory['n'|'u'].H2D   idpy/IdpyCode/IdpyMemory.py:343-425
 *   sclbm_init_populations  InitPopulations + K_InitPopulationsMeta
 *                                           idpy/LBM/MultiPhase.py:1664-1688,
 *                                           idpy/LBM/LBMKernelsMeta.py:282-387
 *   sclbm_init_radial / _flat / _single_flat / _cylinder
 *                           InitRadialInterface, InitFlatInterface, ...
 *                                           idpy/LBM/MultiPhase.py:1771-1937,
 *                                           idpy/LBM/MultiPhaseKernels.py:605-777
 *   sclbm_step              MainLoop / MainLoopMRT step loop (K_ComputeDensityPsiMeta +
 *                           K_ForceCollideStreamSCMP[_MRT]Meta + M_SwapPop per step)
 *                                           idpy/LBM/MultiPhase.py:1015-1097,1311-1402,
 *                                           idpy/IdpyCode/IdpyCode.py:1715-1851
 *   sclbm_compute_moments   ComputeMomentsMeta (+ K_ComputeVelocityAfterForceSCMPMeta)
 *                                           idpy/LBM/MultiPhase.py:1565-1661
 *   sclbm_get_density/_velocity/_populations
 *                           GetDensityField / GetVelocityField / GetPopulations
 *                                           idpy/LBM/LBM.py:634-667
 *   sclbm_check_u           CheckUConvergenceSCMP + K_CheckUMeta
 *                                           idpy/LBM/MultiPhaseLoopChecks.py:96-163,
 *                                           idpy/LBM/LBMKernelsMeta.py:389-498
 *   sclbm_center_of_mass    ComputeCenterOfMass  idpy/LBM/MultiPhase.py:108-137
 *   sclbm_density_at        K_NInNOut (used by DeltaPLaplace) idpy/LBM/LBMKernels.py:506-523
 *   sclbm_set_fluctuations  ShanChenMultiPhase(fluctuations='Gross2011', ...) + CRNGS +
 *                           MainLoopGross2011SRT idpy/LBM/MultiPhase.py:1404-1541,2029-2069,
 *                                           idpy/PRNGS/CRNGS.py:87-337
 *   sclbm_get_seeds         crng.sims_idpy_memory['seeds'].D2H()
 *   sclbm_set_simple        MainLoopSimple* loops  idpy/LBM/MultiPhase.py:164-1014
 *   sclbm_destroy           End()            idpy/LBM/MultiPhase.py:2171-2175
 */
#ifndef SCLBM_H
#define SCLBM_H

#include <stdint.h>

#if defined(__GNUC__)
#define SCLBM_API __attribute__((visibility("default")))
#else
#define SCLBM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SCLBM_OK              0
#define SCLBM_ERR_ARG         1   /* invalid argument (null pointer, bad size, ...) */
#define SCLBM_ERR_UNSUPPORTED 2   /* lattice / stencil / option not built in */
#define SCLBM_ERR_CUDA        3   /* a CUDA runtime call failed */
#define SCLBM_ERR_STATE       4   /* call out of order (e.g. step before init) */
#define SCLBM_ERR_NOMEM       5   /* device allocation failed */
#define SCLBM_ERR_NODEVICE    6   /* no usable sm_100-family device */

/* pseudopotential psi(n) */
#define SCLBM_PSI_EXP_INV       0  /* psi = exp(-1/n)   ('exp(-1./ln_0)')     */
#define SCLBM_PSI_ONE_MINUS_EXP 1  /* psi = 1 - exp(-n) ('(1. - exp(-ln_0))') */
#define SCLBM_PSI_IDENTITY      2  /* psi = n           ('ln_0')              */

/* collision */
#define SCLBM_COLL_BGK 0           /* BGK + Guo forcing, omega = 1/tau */
#define SCLBM_COLL_MRT 1           /* MRT + Guo forcing in the W-orthogonal Hermite basis */

/* storage / arithmetic precision of the populations */
#define SCLBM_FP64         0       /* plain FP64, as the reference */
#define SCLBM_FP32_SHIFTED 1       /* FP32 deviations f_q - w_q*rho0, FP64 reductions */

/* coefficient literals of the expanded collision */
#define SCLBM_LIT_ROUND15 0        /* 15-significant-digit literals, as sympy evalf() emits */
#define SCLBM_LIT_EXACT   1        /* exact coefficients rounded once to double */
#define SCLBM_LIT_FACTORED 2       /* as EXACT; the FP64 BGK step also factors the operator
                                      by opposite directions (fewer FP64 operations, equal up
                                      to rounding; lattices with c2 = 1/3 and symmetric
                                      weights); MRT takes EXACT */

typedef struct sclbm_sim sclbm_sim;

typedef struct sclbm_params {
    int dim;                   /* 2 or 3 */
    int sizes[3];              /* lattice sizes, x first (unused entries ignored) */
    int q;                     /* number of lattice velocities (9: D2Q9, 19: D3Q19) */
    const int *xi;             /* q*dim lattice velocities, in the reference's order */
    const double *w;           /* q lattice weights */
    double c2;                 /* squared sound speed (1/3) */
    int qe;                    /* force-stencil vectors */
    const int *e;              /* qe*dim force-stencil vectors (E4/E6/E8 tables) */
    const double *we;          /* qe force-stencil weights */
    double sc_g;               /* Shan-Chen coupling G */
    int psi_kind;              /* SCLBM_PSI_* */
    int collision;             /* SCLBM_COLL_* */
    double tau;                /* BGK relaxation time (omega = 1/tau) */
    const double *mrt_s;       /* MRT: q*q relaxation matrix S in the moment basis
                                  (row-major; a diagonal S holds the per-moment rates) */
    int precision;             /* SCLBM_FP64 / SCLBM_FP32_SHIFTED */
    double rho0;               /* FP32_SHIFTED: reference density of the shift */
    int literals;              /* SCLBM_LIT_* (FP64 path) */
    int device;                /* CUDA device ordinal */
    /* Optional explicit collision operator, overriding the one built from tau /
     * mrt_s: f*_q = sum_j coll_a[q*q+j] f_j + sum_k coll_b[q*K+k] m_k over the
     * K = sclbm_monomial_count(dim) monomials
     *   [n, n u_a, n u_a u_b (a<=b), F_a, F_a u_b]
     * (how a specific generated reference kernel's printed literals are
     * reproduced exactly).  Both null, or both set. */
    const double *coll_a;
    const double *coll_b;
} sclbm_params;

/* number of collision monomials for a dimension (12 in 2D, 22 in 3D) */
SCLBM_API int sclbm_monomial_count(int dim);

/* library */
SCLBM_API const char *sclbm_version(void);
SCLBM_API const char *sclbm_status_string(int status);
/* message of the last failed call on this thread (empty if none) */
SCLBM_API const char *sclbm_last_error(void);

/* lifetime */
SCLBM_API int sclbm_create(const sclbm_params *p, sclbm_sim **out);
SCLBM_API int sclbm_destroy(sclbm_sim *s);

/* lattice volume and the footprint of the handle in device memory */
SCLBM_API int sclbm_info(const sclbm_sim *s, int64_t *volume, int64_t *device_bytes);

/* fields; host arrays are FP64, x fastest; u as dim planes of volume values */
SCLBM_API int sclbm_set_density(sclbm_sim *s, const double *n);
SCLBM_API int sclbm_set_velocity(sclbm_sim *s, const double *u);
SCLBM_API int sclbm_get_density(sclbm_sim *s, double *n);
SCLBM_API int sclbm_get_velocity(sclbm_sim *s, double *u);
/* populations as q planes of volume values (f_q, not the FP32 deviations) */
SCLBM_API int sclbm_get_populations(sclbm_sim *s, double *pop);
SCLBM_API int sclbm_set_populations(sclbm_sim *s, const double *pop);

/* replace the collision operator (MainLoop <-> MainLoopMRT switch); the
 * populations are kept.  Arguments as the sclbm_params fields of the same name. */
SCLBM_API int sclbm_set_collision(sclbm_sim *s, int collision, double tau, const double *mrt_s,
                                  const double *coll_a, const double *coll_b);

/* initialisation */
SCLBM_API int sclbm_init_populations(sclbm_sim *s);
SCLBM_API int sclbm_init_radial(sclbm_sim *s, double n_g, double n_l, double R, int full_flag);
SCLBM_API int sclbm_init_flat(sclbm_sim *s, double n_g, double n_l, double width, int direction,
                    int full_flag);
SCLBM_API int sclbm_init_single_flat(sclbm_sim *s, double n_g, double n_l, int direction, int full_flag);
SCLBM_API int sclbm_init_cylinder(sclbm_sim *s, double n_g, double n_l, double R, int direction,
                        int full_flag);

/* walls (GetWalls, idpy/LBM/MultiPhase.py:157-162, and then every step as
 * MainLoopWalls, :1226-1309): walls[V] = 1 fluid, 0 wall (2 inlet, 3 outlet for
 * the simple step family, which treats them as neither); psi[V] the psi
 * field, which wall cells keep (their wetting).  From then on density and psi
 * are computed on fluid cells only, the step runs on fluid cells only and a
 * population pushed into a wall returns to the opposite population of its own
 * cell (halfway bounce-back); the two-pass kernels run (no single pass). */
SCLBM_API int sclbm_set_walls(sclbm_sim *s, const int *walls, const double *psi);

/* the reference's "simple" step family (MainLoopSimple, MainLoopSimpleSC,
 * MainLoopSimpleWalls[SC], MainLoopSimpleWallsGravity,
 * MainLoopSimpleWallsInletOutlet[SC]; idpy/LBM/MultiPhase.py:164-1014, kernels
 * idpy/LBM/MultiPhaseKernels.py:132-604, idpy/LBM/LBMKernels.py:117-258,299-456):
 * moments on fluid cells, psi on non-wall cells, an in-place BGK collision with
 * Guo forcing (SCLBM_SIMPLE_GUO) or the Shan-Chen velocity shift
 * (SCLBM_SIMPLE_SC), the periodic stream and halfway bounce-back.  gravity != 0
 * adds g to F_y and collides every non-wall cell (Guo only).  inlet_outlet != 0:
 * wall flags 2 (inlet: n = 2, u = (u_in, 0, ..), equilibrium) and 3 (outlet: the
 * cell at x - 1) are set each step; with SCLBM_SIMPLE_SC the step then streams
 * before it collides, as the reference's loop does.  FP64: the reference's
 * arithmetic in its order (with SCLBM_LIT_ROUND15); FP32_SHIFTED: the same
 * formulas on the shifted storage, mass-conserving.  After steps of this family
 * the density and velocity read back are the arrays the reference's loops leave
 * (the moments at the start of the last step, the stored velocity).
 * use_walls = 0: every cell fluid (MainLoopSimple[SC], which ignore walls).
 * SCLBM_SIMPLE_OFF returns to the generated-kernel step. */
#define SCLBM_SIMPLE_OFF 0
#define SCLBM_SIMPLE_GUO 1
#define SCLBM_SIMPLE_SC  2
SCLBM_API int sclbm_set_simple(sclbm_sim *s, int forcing, int use_walls, int gravity, double g, int inlet_outlet,
                               double u_in);

/* fluctuations: the Gross et al. (2011) fluctuating step
 * (MainLoopGross2011SRT, idpy/LBM/MultiPhase.py:1404-1541; its kernel
 * K_ForceGross2011CollideStreamSCMPMeta, idpy/LBM/MultiPhaseKernelsMeta.py:1369-1557;
 * generators and Box-Muller, idpy/PRNGS/CRNGS.py:603-1276).  Every step adds to
 * population q the noise sum_k coef[q*nr+k] Rm_k (in the reference's print order,
 * the moment names Rm_0, Rm_1, Rm_10, ... sorted as strings), where the nr = q-dim-1
 * random moments are Rm_k = sqrt(m2var[k] log(u0)) cos(2 pi u1), u0, u1 uniform from
 * the cell's congruential generators: generator k drawn twice (indep = 0), or
 * generators 2k and 2k+1 drawn once each (indep = 1, the reference's
 * indep_gaussian).  BGK collision only; not with walls; the two-pass kernels run. */
#define SCLBM_CRNG_NONE   0   /* fluctuations off */
#define SCLBM_CRNG_MINSTD 1   /* Park-Miller 16807 mod 2^31-1 (64-bit product form), uint32 states */
#define SCLBM_CRNG_NUMREC 2   /* x*1664525 + 1013904223 mod 2^32, uint32 states */
#define SCLBM_CRNG_MMIX   3   /* x*6364136223846793005 + 1442695040888963407 mod 2^64, uint64 states */
/* layout of the generator states: seeds[s*V + g] (the reference's 'gpu'
 * ordering, MultiPhase.py:1962-1963) or seeds[s + g*streams] (its 'cpu' one) */
#define SCLBM_SEEDS_STREAM_MAJOR 0
#define SCLBM_SEEDS_CELL_MAJOR   1

/* random moments (q - dim - 1) and generator states per cell (nr or 2 nr) */
SCLBM_API int sclbm_noise_counts(int dim, int q, int indep, int *moments, int *streams);
/* host only: the noise operator GrossShanChenMultiPhase builds
 * (idpy/LBM/Fluctuations.py:40-165) for the lattice, tau and literal mode of p:
 * m2var[nr] = -2 var_k, var_k = norm_k kBT (2 - 1/tau)/tau/c2 n0, and
 * coef[q*nr] = Mw^-1[q][dim+1+k] (Mw the W-orthogonal Hermite basis) */
SCLBM_API int sclbm_noise_operator(const sclbm_params *p, double kBT, double n0, double *m2var, double *coef);
/* switch the fluctuations on (generator SCLBM_CRNG_*) or off (SCLBM_CRNG_NONE).
 * seeds: V * streams initial states (uint32, or uint64 for MMIX) in the given
 * layout.  m2var / coef: null to build the operator from kBT, n0 and the current
 * BGK tau, or the operator to use (e.g. a generated reference kernel's
 * literals).  The operator is kept across sclbm_set_collision; call again after
 * changing tau. */
SCLBM_API int sclbm_set_fluctuations(sclbm_sim *s, int generator, int indep, double kBT, double n0,
                                     const void *seeds, int layout, const double *m2var, const double *coef);
/* the current generator states (crng.sims_idpy_memory['seeds'].D2H()) */
SCLBM_API int sclbm_get_seeds(sclbm_sim *s, void *seeds, int layout);

/* host <-> device transfers of the FP64 field arrays: SCLBM_TRANSFER_AUTO
 * (default) lets a kernel read / write the caller's array directly (converting
 * on the fly) when it is pinned or registered memory or the device can access
 * pageable host memory (Grace-Blackwell NVLink-C2C), else copies through a
 * pinned staging buffer; _STAGED always stages; _DIRECT fails on an array the
 * device cannot access.  Both paths give identical arrays.  pageable_access
 * (optional) reports the device's pageable-memory access. */
#define SCLBM_TRANSFER_AUTO   0
#define SCLBM_TRANSFER_STAGED 1
#define SCLBM_TRANSFER_DIRECT 2
SCLBM_API int sclbm_set_transfer(sclbm_sim *s, int mode, int *pageable_access);

/* time stepping: enqueue nsteps steps on the handle's stream (returns without
 * waiting); sclbm_sync waits for everything enqueued on the handle */
SCLBM_API int sclbm_step(sclbm_sim *s, int64_t nsteps);
SCLBM_API int sclbm_sync(sclbm_sim *s);

/* self-test of the bounded device waits (the mbarrier waits of the staged and
 * mbarrier-ring single-pass variants): one block waits on an mbarrier whose
 * phase cannot complete (two arrivals expected, one made), gives up after
 * `polls` polls (1 .. 2^18, the variants' limit: ~1 s) and returns.  *gave_up: 1
 * when the wait gave up as it must (bit 2: the phase completed, an error);
 * *ms (optional): the launch's duration.  The device stays usable: nothing
 * faults or hangs.  No counterpart in the reference. */
SCLBM_API int sclbm_selftest_bounded_wait(int device, int polls, int *gave_up, double *ms);
/* as sclbm_step, bracketed by CUDA events on the handle's stream; waits and
 * returns the elapsed device time in milliseconds */
SCLBM_API int sclbm_step_timed(sclbm_sim *s, int64_t nsteps, double *ms);
/* per-kernel device time of one step, averaged over nsteps (ms[0]: density+psi
 * pass, ms[1]: fused force+collide+stream pass); kernels are launched one by
 * one, each bracketed by events */
SCLBM_API int sclbm_profile_step(sclbm_sim *s, int64_t nsteps, double *ms, int nms);
/* count of kernels launched by sclbm_step per lattice step */
SCLBM_API int sclbm_kernels_per_step(const sclbm_sim *s, int *count);

/* step path: AUTO = single pass where built (FP32-shifted), else two passes */
#define SCLBM_PATH_AUTO     0  /* the one pass where it applies (paired halo loads where they apply) */
#define SCLBM_PATH_TWO_PASS 1  /* density+psi pass, then force+collide+stream pass */
#define SCLBM_PATH_FUSED    2  /* one pass, psi recomputed in a shared-memory halo ring, one halo cell per load */
/* the one pass with the halo populations loaded two x-adjacent cells per load
 * (3D lattices with even Lx and an E6/E8 stencil; otherwise as SCLBM_PATH_FUSED) */
#define SCLBM_PATH_FUSED_PAIRS 3
/* choose the step path and the marching chunk (planes per work item, 0 = planned) */
SCLBM_API int sclbm_set_tuning(sclbm_sim *s, int path, int chunk);
SCLBM_API int sclbm_get_tuning(const sclbm_sim *s, int *path, int *chunk, int *grid);

/* Staging of the 3D paired single pass (flags; FP32 BGK, E6/E8, even Lx).  No
 * counterpart in the reference (its generated kernels use a fixed 128-thread
 * block, idpy/LBM/MultiPhase.py:2072-2085).  The results are bit-identical
 * with and without staging.
 *   SCLBM_STAGE_HALO_ASYNC  halo populations of the next plane copied into
 *                           shared memory with cp.async while a plane collides
 *   SCLBM_STAGE_OWN_TMA     the tile's own populations of the next plane loaded
 *                           by one TMA box per plane (needs Lx % 4 == 0) */
#define SCLBM_STAGE_HALO_ASYNC 1
#define SCLBM_STAGE_OWN_TMA 2
/* the kernel configuration of a handle's step: path (SCLBM_PATH_*), chunk
 * (planes per work item, 0 = planned), staging (SCLBM_STAGE_* flags, -1 =
 * automatic), tile (tile shape of the 3D paired single pass, FP32 BGK
 * without walls or noise: 0 = 32x8, 1 = 64x8, 2 = 32x16, 3 = 128x8, 4 = 32x8
 * with streaming (evict-first) stores, 5 = 32x8 with an mbarrier per psi
 * plane in place of the per-plane block barrier; -1 = automatic; staging applies to
 * shape 0 only), order (of the single pass's work items over the grid: 0 x
 * fastest, 1 the chunk fastest, 2 y fastest; -1 = automatic), grid (CTAs
 * launched; output only).  get reports what runs: the path, staging, tile and
 * order that apply to this handle.  Every variant computes bit-identical
 * results. */
typedef struct sclbm_tuning {
    int path;
    int chunk;
    int staging;
    int tile;
    int order;
    int grid;
} sclbm_tuning;
SCLBM_API int sclbm_set_tuning_ex(sclbm_sim *s, const sclbm_tuning *t);
SCLBM_API int sclbm_get_tuning_ex(const sclbm_sim *s, sclbm_tuning *t);

/* Autotuner.  No counterpart in the reference (fixed 128-thread blocks,
 * idpy/LBM/MultiPhase.py:2072-2085).  Times every variant of the handle's
 * current step that computes bit-identical results (single pass: one or two
 * halo cells per load, the staging flags, the chunk length, i.e. the cells
 * each thread marches; the two-pass path has none) with CUDA events over
 * trial_steps launches on the handle's stream, applies the fastest and caches
 * it for the handle's key (lattice, stencil, operator, precision, walls, box,
 * device SM count); handles created later with that key on the automatic
 * choice (path AUTO, chunk 0, staging -1) use it.  The trial launches all read
 * the current populations, so the simulation state is unchanged.  best (may be
 * NULL) gets the configuration, *best_ms (may be NULL) its time per step.
 * Fluctuating handles (a trial would advance their generators) and the simple
 * step family (its inlet/outlet kernels write the current populations) are
 * refused with SCLBM_ERR_UNSUPPORTED. */
SCLBM_API int sclbm_autotune(sclbm_sim *s, int trial_steps, sclbm_tuning *best, double *best_ms);
SCLBM_API int sclbm_clear_tuning_cache(void);

/* observables */
SCLBM_API int sclbm_compute_moments(sclbm_sim *s);
/* sum of all populations (FP64 accumulation) and total momentum sum_q xi_q f_q */
SCLBM_API int sclbm_reductions(sclbm_sim *s, double *mass, double *momentum);
/* CheckUConvergenceSCMP on the last compute_moments velocity:
 * u_conv = sum_cells sum_d |u - u_old| / V, max_u = sqrt(max |u|^2 / c2); then
 * u_old = u.  The first call compares against zero, as the reference does. */
SCLBM_API int sclbm_check_u(sclbm_sim *s, double *u_conv, double *max_u);
/* mass and centre of mass sum(n x_d)/sum(n) from the density field */
SCLBM_API int sclbm_center_of_mass(sclbm_sim *s, double *mass, double *cm);
/* density at count linear cell indices */
SCLBM_API int sclbm_density_at(sclbm_sim *s, const int64_t *idx, int count, double *out);
/* 1 if every density value is finite, else 0 (max |n| also returned) */
SCLBM_API int sclbm_density_finite(sclbm_sim *s, int *finite, double *max_abs);
/* Mass restoring: *before = the FP64 mass of the current populations; if
 * target is finite, (target - mass) / V is then added to the rest population
 * of every cell.  FP32-shifted storage rounds every stored population, and in
 * a near-steady state the same rounding repeats every step, so the mass drifts
 * linearly (about 1e-9 relative per step); a caller that checks convergence
 * every K steps restores the initial mass there.  No counterpart in the
 * reference, whose FP64 step conserves mass to round-off. */
SCLBM_API int sclbm_restore_mass(sclbm_sim *s, double target, double *before);

/* ---------------------------------------------------------------------------
 * Batches: many independent periodic lattices of different sizes (ragged
 * droplet sweeps), FP32-shifted storage, stepped together by one launch per
 * step (CTAs take work items from a device queue, so retired lattices cost
 * nothing).  No counterpart in the reference, which runs one
 * ShanChenMultiPhase object per droplet (idpy/LBM/MultiPhase.py:140); each
 * lattice follows the same step as sclbm_step.
 * ------------------------------------------------------------------------- */
typedef struct sclbm_batch sclbm_batch;

/* p gives the lattice, stencil, psi, collision and device (sizes, sc_g and
 * rho0 unused; precision must be SCLBM_FP32_SHIFTED); lattice i has sizes
 * sizes[i*dim ..], coupling G[i] and shift rho0[i]. */
SCLBM_API int sclbm_batch_create(const sclbm_params *p, int n, const int *sizes, const double *G,
                                 const double *rho0, sclbm_batch **out);
SCLBM_API int sclbm_batch_destroy(sclbm_batch *b);
/* total cells and device bytes */
SCLBM_API int sclbm_batch_info(const sclbm_batch *b, int64_t *cells, int64_t *device_bytes);
/* density of lattice i (its own x-fastest layout); velocity starts at zero */
SCLBM_API int sclbm_batch_set_density(sclbm_batch *b, int i, const double *n);
SCLBM_API int sclbm_batch_get_density(sclbm_batch *b, int i, double *n);
/* equilibrium populations of every lattice from its density (u = 0) */
SCLBM_API int sclbm_batch_init_populations(sclbm_batch *b);
/* equilibrium populations (u = 0) of active lattice i alone from the density
 * last given by sclbm_batch_set_density (a restart of one lattice, e.g. a
 * warm start that is replaced by a cold start) */
SCLBM_API int sclbm_batch_init_lattice(sclbm_batch *b, int i);
/* enqueue nsteps steps of every active lattice (returns without waiting) */
SCLBM_API int sclbm_batch_step(sclbm_batch *b, int64_t nsteps);
SCLBM_API int sclbm_batch_step_timed(sclbm_batch *b, int64_t nsteps, double *ms);
/* per active lattice: u_conv (sum |u - u_old| / V since the last check, the
 * reference's CheckUConvergenceSCMP measure), max_u = sqrt(max|u|^2 / c2) and
 * mass (FP64 reductions); u_old is then updated.  Retired lattices keep their
 * last values. */
SCLBM_API int sclbm_batch_check(sclbm_batch *b, double *u_conv, double *max_u, double *mass);
/* retire (0) or keep (1) lattices; a retired lattice is no longer stepped */
SCLBM_API int sclbm_batch_set_active(sclbm_batch *b, const int *active);
/* steps each lattice has taken */
SCLBM_API int sclbm_batch_steps(const sclbm_batch *b, int64_t *steps);
/* sclbm_restore_mass per active lattice: before[i] = its FP64 mass; where
 * target[i] is finite, (target[i] - mass) / V_i is added to its rest
 * populations. */
SCLBM_API int sclbm_batch_restore_mass(sclbm_batch *b, const double *target, double *before);
/* density (FP64 sum of the populations) at the centre cell (L_d / 2 in every
 * dimension) and at the last cell of every active lattice: the two densities
 * of DeltaPLaplace (idpy/LBM/MultiPhase.py:1690-1757, K_NInNOut
 * idpy/LBM/LBMKernels.py:506-523).  Retired lattices keep their last values. */
SCLBM_API int sclbm_batch_probe(sclbm_batch *b, double *n_in, double *n_out);
/* make sclbm_batch_probe return the mean density over the cube (square in 2D)
 * of side 2 rad + 1 about each probe cell, rad in [0, 4] (0, the default: the
 * single cell, as the reference's DeltaPLaplace reads them).  A block mean
 * lowers the FP32 rounding noise of a single probe cell; in equilibrium the
 * bulk cells agree, but spurious-current structure near the droplet centre
 * biases the mean by ~1e-5 of the Laplace pressure, so the sweeps keep single
 * cells.  No counterpart in the reference. */
SCLBM_API int sclbm_batch_set_probe_radius(sclbm_batch *b, int rad);
/* tile width of a 2D batch's work items: 0 (the default, the single-lattice
 * kernel's 256 cells) or 64 (four times as many items of a quarter the width,
 * for batches whose lattices are too few or too small to fill the GPU with
 * 256-cell rows).  The results are bit-identical.  3D batches take 0 only.
 * No counterpart in the reference. */
SCLBM_API int sclbm_batch_set_tile_width(sclbm_batch *b, int tx);
/* on (the default): each cell's rest population absorbs the rounding errors
 * of its density sum and of the subtraction chain (compensated sums), so the
 * stored FP32 populations conserve mass to one rounding per cell and step;
 * off: plain FP32 sums, ~11 % shorter steps, mass drift left to
 * sclbm_batch_restore_mass.  Off is built for 3D batches with paired halo
 * loads only (SCLBM_ERR_UNSUPPORTED otherwise).  No counterpart in the
 * reference. */
SCLBM_API int sclbm_batch_set_mass_compensation(sclbm_batch *b, int on);

/* ---------------------------------------------------------------------------
 * Warm-start surrogate: an MLP 5 -> 64 -> 64 -> 64 -> 1 with SiLU, BF16
 * parameters (FP32 master copy) and FP32 accumulation, trained with Adam on
 * (input, target) pairs the caller gives (normalised features of a droplet
 * and a radial position -> normalised density).  No counterpart in the
 * reference, which starts every droplet from a tanh profile.  Parameters are
 * one float vector of sclbm_mlp_param_count() values:
 * W1[64][5], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], W4[64], b4.
 * ------------------------------------------------------------------------- */
typedef struct sclbm_mlp sclbm_mlp;
SCLBM_API int sclbm_mlp_param_count(int *count);
/* weights and biases uniform in +-1/sqrt(fan_in) from the seed */
SCLBM_API int sclbm_mlp_create(int device, uint64_t seed, sclbm_mlp **out);
SCLBM_API int sclbm_mlp_destroy(sclbm_mlp *m);
/* FP32 master parameters; setting them also resets the Adam state and step */
SCLBM_API int sclbm_mlp_set_params(sclbm_mlp *m, const float *w);
SCLBM_API int sclbm_mlp_get_params(sclbm_mlp *m, float *w);
/* training set: n inputs x[n][5] and targets t[n] (copied to the device) */
SCLBM_API int sclbm_mlp_set_data(sclbm_mlp *m, int64_t n, const float *x, const float *t);
/* steps of Adam (beta 0.9 / 0.999, eps 1e-8) on the mean squared error of
 * `batch` samples drawn on the device per step; loss[steps] (optional) gets
 * the loss of every step */
SCLBM_API int sclbm_mlp_train(sclbm_mlp *m, int64_t steps, int64_t batch, float lr, float *loss);
/* gradient of the mean squared error over the n given samples with the
 * current parameters (no update): grad[param_count], *loss */
SCLBM_API int sclbm_mlp_gradient(sclbm_mlp *m, int64_t n, const float *x, const float *t, float *grad,
                                 float *loss);
/* outputs y[n] for inputs x[n][5] */
SCLBM_API int sclbm_mlp_predict(sclbm_mlp *m, int64_t n, const float *x, float *y);

/* ---------------------------------------------------------------------------
 * One step that allocates no device memory.  No counterpart in the reference.
 *
 * For callers that cannot let this library call cudaMalloc: a host program
 * that reserves its whole device-memory budget once, in its own pool, and has
 * no way to hand a handle's allocations to it; or a service in which an
 * allocation or free during stepping (cudaFree synchronizes the device) would
 * stall its other streams.  Such a caller keeps the populations in buffers it
 * already owns and calls this instead of sclbm_create + sclbm_step.
 *
 * p describes the lattice exactly as for sclbm_create (sizes, stencils, G,
 * psi, collision, precision, rho0, literals, device).  pop_in and pop_out are
 * device pointers to q * V values each, q-major with x fastest, in the
 * storage of p->precision (FP64: f; FP32_SHIFTED: float f - w_q rho0); they
 * must not overlap.  One call enqueues one step (the density+psi pass and the
 * force+collide+stream pass, the same kernels as a handle on
 * SCLBM_PATH_TWO_PASS) on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and returns without waiting; the caller swaps the buffers between
 * calls.
 *
 * The scratch between the two passes (density and psi) is a fixed array in
 * the library's device data, 16 MiB, held on every GPU that loads the library
 * until the process exits.  Lattices of more than SCLBM_NOALLOC_MAX_CELLS
 * cells are rejected with SCLBM_ERR_ARG.  All calls on one device share that
 * device's copy of the array, which keeps the last call's contents, so calls
 * whose kernels overlap on the GPU (streams with no ordering between them)
 * race: order them on one stream.  The first
 * call on each device looks up the array's device address in the context
 * current on the calling thread (set-up done once per device and context);
 * a later call that finds another context current (after a cudaDeviceReset,
 * or with a context the caller made current) looks it up again, since the
 * array then sits at another address.  Make the first call in each context
 * before any stream capture.  A CUDA error already pending on the calling
 * thread when the call starts is reported (SCLBM_ERR_CUDA) and left uncleared,
 * and nothing is enqueued.
 * ------------------------------------------------------------------------- */
#define SCLBM_NOALLOC_MAX_CELLS (1 << 20)
SCLBM_API int sclbm_step_noalloc(const sclbm_params *p, const void *pop_in, void *pop_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SCLBM_H */
