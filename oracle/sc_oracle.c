/*
 * CPU oracle for the Shan-Chen multiphase LBM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the arithmetic of
 * the reference's CTypes FP64 path (lullimat/idea.deploy, package idpy) so the
 * CUDA path can be checked against it.  Only tests/, the smoke check and the
 * CPU-baseline leg of bench.py may load it; the product never does.
 *
 * Layout follows the reference's 'cpu' ordering: pop[q + g*Q], u[d + g*D],
 * g = x + L0*(y + L1*z) (idpy/LBM/LBM.py:529-537).
 *
 * The collision is driven by term tables built in oracle.py: for every
 * population q a list of terms ((coef * x1) * x2) * x3 summed left to right,
 * where x_i index the per-cell value vector
 *      v = [n, u_0..u_{D-1}, F_0..F_{D-1}, f_0..f_{Q-1}].
 * That is exactly how the generated C of the reference evaluates each
 * post-collision population (idpy/LBM/Collisions.py:251-316 emits the
 * expanded sympy expression; terms appear in sympy's print order), so with
 * the reference's own literals the oracle is bit-identical to it.
 *
 * Reference kernels restated here:
 *   K_ComputeDensityPsiMeta               idpy/LBM/MultiPhaseKernelsMeta.py:107-167
 *   K_ForceCollideStreamSCMPMeta          idpy/LBM/MultiPhaseKernelsMeta.py:169-345
 *   K_ForceCollideStreamSCMP_MRTMeta      idpy/LBM/MultiPhaseKernelsMeta.py:891-1075
 *   K_ComputeVelocityAfterForceSCMPMeta   idpy/LBM/MultiPhaseKernelsMeta.py:1077-1219
 *   K_InitPopulationsMeta                 idpy/LBM/LBMKernelsMeta.py:282-387
 *   SC force (gradient) codegen           idpy/LBM/IDShanChenForce.py:44-116,
 *                                         idpy/IdpyStencils/IdpyStencils.py:1431-1596
 *   periodic neighbour wrap               idpy/IdpyCode/IdpyUnroll.py:37-48
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

#define ORC_MAXQ 27
#define ORC_MAXT 64

enum { ORC_PSI_EXP_INV = 0, ORC_PSI_ONE_MINUS_EXP = 1, ORC_PSI_IDENTITY = 2 };

typedef struct {
    int dim;          /* 2 or 3 */
    int L[3];         /* sizes, x first */
    int Q;            /* lattice populations */
    int QE;           /* force-stencil vectors */
    const int *xi;    /* Q*dim lattice velocities */
    const int *e;     /* QE*dim force-stencil vectors */
    const double *we; /* QE force-stencil weights (double, as the caller gives them) */
    double G;         /* Shan-Chen coupling */
    int psi_kind;
    /* collision terms: for q, terms [t_off[q], t_off[q+1]) */
    const int *t_off;      /* Q+1 */
    const double *t_coef;  /* T */
    const int *t_nf;       /* T: factors (0..3) */
    const int *t_fid;      /* 3*T factor ids into v */
    /* velocity sums, per d: signed population list in order */
    const int *v_off;      /* D+1 */
    const int *v_pop;      /* population index */
    const int *v_sign;     /* +1 / -1 */
    /* density sum order */
    const int *n_order;    /* Q */
} orc_cfg;

static inline int wrap(int x, int L) {
    /* branch-free periodic wrap for |offset| < L, as in the reference macros */
    if (x >= L) return x - L;
    if (x < 0) return x + L;
    return x;
}

static inline double psi_of(int kind, double n) {
    switch (kind) {
    case ORC_PSI_EXP_INV: return exp(-1. / n);
    case ORC_PSI_ONE_MINUS_EXP: return (1. - exp(-n));
    default: return n;
    }
}

static inline void coords(const orc_cfg *c, long g, int *x) {
    x[0] = (int)(g % c->L[0]);
    if (c->dim == 2) {
        x[1] = (int)(g / c->L[0]);
        x[2] = 0;
    } else {
        x[1] = (int)((g / c->L[0]) % c->L[1]);
        x[2] = (int)(g / ((long)c->L[0] * c->L[1]));
    }
}

static inline long index_of(const orc_cfg *c, const int *x) {
    long g = x[0];
    g += (long)c->L[0] * x[1];
    if (c->dim == 3) g += (long)c->L[0] * c->L[1] * x[2];
    return g;
}

static inline long neighbour(const orc_cfg *c, const int *x, const int *off) {
    int y[3] = {0, 0, 0};
    for (int d = 0; d < c->dim; d++) y[d] = wrap(x[d] + off[d], c->L[d]);
    return index_of(c, y);
}

static long volume(const orc_cfg *c) {
    long V = 1;
    for (int d = 0; d < c->dim; d++) V *= c->L[d];
    return V;
}

/* n = sum_q f_q (reference print order), psi = psi(n) */
int orc_density_psi(const orc_cfg *c, const double *pop, double *n, double *psi) {
    const long V = volume(c);
    const int Q = c->Q;
    for (long g = 0; g < V; g++) {
        const double *f = pop + g * Q;
        double s = f[c->n_order[0]];
        for (int i = 1; i < Q; i++) s = s + f[c->n_order[i]];
        psi[g] = psi_of(c->psi_kind, s);
        n[g] = s;
    }
    return 0;
}

/* F_d = -G psi(x) sum_a w_a e_{a,d} psi(x+e_a), accumulated as the reference does */
static void sc_force(const orc_cfg *c, const double *psi, long g, const int *x, double *F) {
    double dp[3] = {0., 0., 0.};
    for (int a = 0; a < c->QE; a++) {
        const int *e = c->e + a * c->dim;
        const long nb = neighbour(c, x, e);
        const double p = psi[nb];
        for (int d = 0; d < c->dim; d++) {
            if (e[d] == 0) continue;
            const double w = (double)abs(e[d]) * c->we[a];
            if (e[d] > 0) dp[d] += w * p;
            else dp[d] -= w * p;
        }
    }
    const double s = -c->G * psi[g];
    for (int d = 0; d < c->dim; d++) F[d] = dp[d] * s;
}

/* u_d = (sum_q xi_{q,d} f_q)/n, then u_d += 0.5*F_d/n (Guo shift) */
static void velocity(const orc_cfg *c, const double *f, double n, const double *F, double *u) {
    for (int d = 0; d < c->dim; d++) {
        double s = 0.;
        int first = 1;
        for (int k = c->v_off[d]; k < c->v_off[d + 1]; k++) {
            const double t = c->v_sign[k] > 0 ? f[c->v_pop[k]] : -f[c->v_pop[k]];
            if (first) { s = t; first = 0; }
            else s = s + t;
        }
        u[d] = s / n;
        u[d] += 0.5 * F[d] / n;
    }
}

static inline double eval_terms(const orc_cfg *c, int q, const double *v) {
    double acc = 0.;
    int first = 1;
    for (int t = c->t_off[q]; t < c->t_off[q + 1]; t++) {
        double p = c->t_coef[t];
        const int nf = c->t_nf[t];
        for (int k = 0; k < nf; k++) p = p * v[c->t_fid[3 * t + k]];
        if (first) { acc = p; first = 0; }
        else acc = acc + p;
    }
    return acc;
}

/* One fused force + collision + push-stream pass: pop -> pop_swap */
int orc_force_collide_stream(const orc_cfg *c, const double *pop, const double *n,
                             const double *psi, double *pop_swap) {
    const long V = volume(c);
    const int Q = c->Q, D = c->dim;
    double v[1 + 6 + ORC_MAXQ];
    for (long g = 0; g < V; g++) {
        int x[3];
        coords(c, g, x);
        double F[3];
        sc_force(c, psi, g, x, F);
        const double *f = pop + g * Q;
        double u[3];
        velocity(c, f, n[g], F, u);
        v[0] = n[g];
        for (int d = 0; d < D; d++) { v[1 + d] = u[d]; v[1 + D + d] = F[d]; }
        for (int q = 0; q < Q; q++) v[1 + 2 * D + q] = f[q];
        for (int q = 0; q < Q; q++) {
            const long dst = neighbour(c, x, c->xi + q * D);
            pop_swap[q + dst * Q] = eval_terms(c, q, v);
        }
    }
    return 0;
}

/* ComputeMomentsMeta second kernel: writes n (unchanged) and the shifted u */
int orc_velocity_after_force(const orc_cfg *c, const double *pop, const double *n,
                             const double *psi, double *u_out) {
    const long V = volume(c);
    const int Q = c->Q, D = c->dim;
    for (long g = 0; g < V; g++) {
        int x[3];
        coords(c, g, x);
        double F[3], u[3];
        sc_force(c, psi, g, x, F);
        velocity(c, pop + g * Q, n[g], F, u);
        for (int d = 0; d < D; d++) u_out[d + g * D] = u[d];
    }
    return 0;
}

/* Equilibrium populations from (n, u): same term tables, products formed first
 * (the reference precomputes n*u_a and n*u_a*u_b, LBMKernelsMeta.py:282-387). */
int orc_init_populations(const orc_cfg *c, const double *n, const double *u, double *pop) {
    const long V = volume(c);
    const int Q = c->Q, D = c->dim;
    double v[1 + 6 + ORC_MAXQ];
    for (long g = 0; g < V; g++) {
        v[0] = n[g];
        for (int d = 0; d < D; d++) { v[1 + d] = u[d + g * D]; v[1 + D + d] = 0.; }
        for (int q = 0; q < Q; q++) {
            double acc = 0.;
            int first = 1;
            for (int t = c->t_off[q]; t < c->t_off[q + 1]; t++) {
                const int nf = c->t_nf[t];
                double p = 1.;
                if (nf > 0) {
                    p = v[c->t_fid[3 * t]];
                    for (int k = 1; k < nf; k++) p = p * v[c->t_fid[3 * t + k]];
                }
                p = c->t_coef[t] * p;
                if (first) { acc = p; first = 0; }
                else acc = acc + p;
            }
            pop[q + g * Q] = acc;
        }
    }
    return 0;
}

/* nsteps of MainLoop: density/psi, fused step, swap (IdpyLoop.Run).  On return
 * the current populations are in *pop_a (buffers are swapped as needed). */
int orc_run(const orc_cfg *c, double *pop_a, double *pop_b, double *n, double *psi,
            int nsteps, int *swapped) {
    double *cur = pop_a, *nxt = pop_b;
    for (int s = 0; s < nsteps; s++) {
        orc_density_psi(c, cur, n, psi);
        orc_force_collide_stream(c, cur, n, psi, nxt);
        double *t = cur; cur = nxt; nxt = t;
    }
    *swapped = (cur != pop_a);
    return 0;
}

/* ---- walls (GetWalls / MainLoopWalls, idpy/LBM/MultiPhase.py:157-162,1226-1309) ----
 * walls[g] = 1 fluid, 0 wall.  Density and psi are computed on fluid cells only
 * (K_ComputeDensityPsiWallsMeta, MultiPhaseKernelsMeta.py:42-105); wall cells keep
 * the psi they were given.  The fused step runs on fluid cells only and, for
 * q != 0, pushes into the opposite population of the same cell when the target
 * is a wall (SRTCollisionPlusGuoPushStreamWallsCode, Collisions.py:705-860). */
int orc_density_psi_walls(const orc_cfg *c, const double *pop, const int *walls, double *n, double *psi) {
    const long V = volume(c);
    const int Q = c->Q;
    for (long g = 0; g < V; g++) {
        if (walls[g] != 1) continue;
        const double *f = pop + g * Q;
        double s = f[c->n_order[0]];
        for (int i = 1; i < Q; i++) s = s + f[c->n_order[i]];
        psi[g] = psi_of(c->psi_kind, s);
        n[g] = s;
    }
    return 0;
}

int orc_force_collide_stream_walls(const orc_cfg *c, const double *pop, const double *n, const double *psi,
                                   const int *walls, const int *opposite, double *pop_swap) {
    const long V = volume(c);
    const int Q = c->Q, D = c->dim;
    double v[1 + 6 + ORC_MAXQ];
    for (long g = 0; g < V; g++) {
        if (walls[g] != 1) continue;
        int x[3];
        coords(c, g, x);
        double F[3];
        sc_force(c, psi, g, x, F);
        const double *f = pop + g * Q;
        double u[3];
        velocity(c, f, n[g], F, u);
        v[0] = n[g];
        for (int d = 0; d < D; d++) { v[1 + d] = u[d]; v[1 + D + d] = F[d]; }
        for (int q = 0; q < Q; q++) v[1 + 2 * D + q] = f[q];
        for (int q = 0; q < Q; q++) {
            long dst = neighbour(c, x, c->xi + q * D);
            int qd = q;
            if (q != 0 && walls[dst] == 0) {
                dst = g;
                qd = opposite[q];
            }
            pop_swap[qd + dst * Q] = eval_terms(c, q, v);
        }
    }
    return 0;
}

int orc_run_walls(const orc_cfg *c, double *pop_a, double *pop_b, double *n, double *psi, const int *walls,
                  const int *opposite, int nsteps, int *swapped) {
    double *cur = pop_a, *nxt = pop_b;
    for (int s = 0; s < nsteps; s++) {
        orc_density_psi_walls(c, cur, walls, n, psi);
        orc_force_collide_stream_walls(c, cur, n, psi, walls, opposite, nxt);
        double *t = cur; cur = nxt; nxt = t;
    }
    *swapped = (cur != pop_a);
    return 0;
}

/* ---- fluctuations (Gross et al. 2011, MainLoopGross2011SRT, idpy/LBM/MultiPhase.py:1404-1541) ----
 * K_ForceGross2011CollideStreamSCMPMeta (idpy/LBM/MultiPhaseKernelsMeta.py:1369-1557) is the
 * BGK + Guo push step with, for every population q, the terms coef * Rm_k added one by one
 * after the collided value (Collisions.py:526-527), where Rm_k are Gaussian random moments:
 *   Rm_k = sqrt(-2 var_k log(u0)) cos(TWOPI u1) + 0        (CRNGS.py:924-1058)
 * u0, u1 uniform in [0, 1] from congruential generators (CRNGS.py:603-735): one stream per
 * moment drawn twice, or (independent mode) streams 2k and 2k+1 drawn once each.  Generator
 * states are read at the start of the cell update and written back at its end
 * (CRNGS.py:1061-1113).  seeds[s + g * ns], the reference's CPU ordering
 * (MultiPhase.py:1964-1965); 32-bit generators keep their state in the low 32 bits. */
enum { ORC_CRNG_MINSTD = 1, ORC_CRNG_NUMREC = 2, ORC_CRNG_MMIX = 3 };

typedef struct {
    int kind;              /* ORC_CRNG_* */
    int indep;             /* 0: one stream per moment, 1: two */
    int nr;                /* random moments, Q - (D + 1) */
    const double *m2var;   /* nr: -2 * variance (the product the generated C folds) */
    const int *t_off;      /* Q+1: noise terms of population q in [t_off[q], t_off[q+1]) */
    const int *t_mom;      /* moment of each term */
    const double *t_coef;  /* literal of each term */
} orc_noise;

static const double ORC_TWOPI = 6.283185307179586;  /* 2. * np.pi, the reference's TWOPI */

/* one step of the generator (MMIX CRNGS.py:717-731, NUMREC :705-715, MINSTD 64-bit :674-703) */
static inline uint64_t crng_next(int kind, uint64_t s) {
    if (kind == ORC_CRNG_MMIX) return s * 6364136223846793005ULL + 1442695040888963407ULL;
    if (kind == ORC_CRNG_NUMREC) return (uint32_t)((uint32_t)s * 1664525U + 1013904223U);
    const uint64_t sw = 16807ULL * (uint32_t)s;
    uint32_t r = (uint32_t)((sw & 0x7fffffffULL) + (sw >> 31));
    if (r & 0x80000000U) r = (r & 0x7fffffffU) + 1U;
    return r;
}

/* ((PopType)seed) / ((PopType)ID_RANDMAX_<kind>)  (CRNGS.py:737-773) */
static inline double crng_flat(int kind, uint64_t s) {
    if (kind == ORC_CRNG_MMIX) return (double)s / 18446744073709551616.0;  /* (double)(2^64 - 1) */
    if (kind == ORC_CRNG_NUMREC) return (double)(uint32_t)s / 4294967295.0;
    return (double)(uint32_t)s / 2147483647.0;
}

int orc_force_collide_stream_noise(const orc_cfg *c, const orc_noise *z, const double *pop, const double *n,
                                   const double *psi, uint64_t *seeds, double *pop_swap) {
    const long V = volume(c);
    const int Q = c->Q, D = c->dim, ns = z->indep ? 2 * z->nr : z->nr;
    double v[1 + 6 + ORC_MAXQ];
    double rm[ORC_MAXQ];
    for (long g = 0; g < V; g++) {
        int x[3];
        coords(c, g, x);
        double F[3];
        sc_force(c, psi, g, x, F);
        const double *f = pop + g * Q;
        double u[3];
        velocity(c, f, n[g], F, u);
        uint64_t *sd = seeds + g * ns;
        for (int k = 0; k < z->nr; k++) {
            double u0, u1;
            if (z->indep) {
                sd[2 * k] = crng_next(z->kind, sd[2 * k]);
                u0 = crng_flat(z->kind, sd[2 * k]);
                sd[2 * k + 1] = crng_next(z->kind, sd[2 * k + 1]);
                u1 = crng_flat(z->kind, sd[2 * k + 1]);
            } else {
                sd[k] = crng_next(z->kind, sd[k]);
                u0 = crng_flat(z->kind, sd[k]);
                sd[k] = crng_next(z->kind, sd[k]);
                u1 = crng_flat(z->kind, sd[k]);
            }
            rm[k] = sqrt(z->m2var[k] * log(u0)) * cos(ORC_TWOPI * u1) + 0.;
        }
        v[0] = n[g];
        for (int d = 0; d < D; d++) { v[1 + d] = u[d]; v[1 + D + d] = F[d]; }
        for (int q = 0; q < Q; q++) v[1 + 2 * D + q] = f[q];
        for (int q = 0; q < Q; q++) {
            const long dst = neighbour(c, x, c->xi + q * D);
            double acc = eval_terms(c, q, v);
            for (int t = z->t_off[q]; t < z->t_off[q + 1]; t++) acc = acc + z->t_coef[t] * rm[z->t_mom[t]];
            pop_swap[q + dst * Q] = acc;
        }
    }
    return 0;
}

int orc_run_noise(const orc_cfg *c, const orc_noise *z, double *pop_a, double *pop_b, double *n, double *psi,
                  uint64_t *seeds, int nsteps, int *swapped) {
    double *cur = pop_a, *nxt = pop_b;
    for (int s = 0; s < nsteps; s++) {
        orc_density_psi(c, cur, n, psi);
        orc_force_collide_stream_noise(c, z, cur, n, psi, seeds, nxt);
        double *t = cur; cur = nxt; nxt = t;
    }
    *swapped = (cur != pop_a);
    return 0;
}

/* ---- the "simple" step family (MainLoopSimple*, idpy/LBM/MultiPhase.py:164-1014) ----
 * Hand-written kernels over q-major arrays (pop[g + q*V], u[g + d*V]), run in this order
 * each step (IdpyLoop.Run, serial on the CTypes backend):
 *   inlet   K_SetPopNUXInletDutyCycle   LBMKernels.py:299-357   (walls == 2: n = 2, u = (u_in, 0..), equilibrium)
 *   outlet  K_SetPopNUOutletNoGradient  LBMKernels.py:423-456   (walls == 3: n, u, pop of the cell at x - 1)
 *   moments K_ComputeMoments[Walls]     LBMKernels.py:187-258   (walls == 1)
 *   psi     K_ComputePsi[Walls]         MultiPhaseKernels.py:562-604 (walls != 0)
 *   collide K_Collision_ShanChen[Guo]MultiPhase[Walls][Gravity]  MultiPhaseKernels.py:132-561
 *           in place, Guo forcing or the Shan-Chen velocity shift; gravity adds g to F_y
 *           (and that kernel collides every cell with walls != 0)
 *   stream  K_StreamPeriodic (pull)     LBMKernels.py:117-149
 *   bounce  K_HalfWayBounceBack         LBMKernels.py:151-185  (walls == 0)
 * MainLoopSimpleWallsInletOutletSC (MultiPhase.py:735-887) runs them in another order:
 * outlet, inlet, stream, bounce, swap, moments, psi, collide (the step ends after the
 * collision) -- order 1 below.
 * Every expression keeps the reference's operand order; CM2 = 3.0, CM4 = 9.0. */
typedef struct {
    int dim, L[3], Q, QE;
    const int *xi;        /* Q*dim */
    const double *w;      /* Q */
    const int *e;         /* QE*dim */
    const double *we;     /* QE */
    const int *opposite;  /* Q */
    double G, omega;
    int psi_kind;
    int forcing;          /* 0 Guo, 1 Shan-Chen velocity shift */
    int gravity;          /* 1: F_y += g and collide walls != 0 */
    double g;
    int inout;            /* 1: inlet (walls 2) and outlet (walls 3) setters */
    double u_in;
    int order;            /* 0: set, moments, psi, collide, stream, bounce; 1: the SC inlet/outlet order */
} orc_simple;

static inline void s_pos(const orc_simple *c, long g, int *p) {
    p[0] = (int)(g % c->L[0]);
    if (c->dim > 1) p[1] = (int)((g / c->L[0]) % c->L[1]);
    if (c->dim > 2) p[2] = (int)(g / ((long)c->L[0] * c->L[1]));
}
static inline long s_index(const orc_simple *c, const int *p) {
    long i = p[0];
    if (c->dim > 1) i += (long)p[1] * c->L[0];
    if (c->dim > 2) i += (long)p[2] * c->L[0] * c->L[1];
    return i;
}

static void s_inlet(const orc_simple *c, long V, double *pop, double *n, double *u, const int *walls) {
    const int D = c->dim, Q = c->Q;
    for (long g = 0; g < V; g++) {
        if (walls[g] != 2) continue;
        const double ln = n[g] = 2.;
        const double u_swap = c->u_in;
        double lu[3];
        const double u_dot_u = u_swap * u_swap;
        lu[0] = u[g] = u_swap;
        for (int d = 1; d < D; d++) lu[d] = u[g + d * V] = 0.;
        for (int q = 0; q < Q; q++) {
            double u_dot_xi = 0.;
            for (int d = 0; d < D; d++) u_dot_xi += lu[d] * c->xi[d + q * D];
            double leq = 1.;
            leq += u_dot_xi * 3.0;
            leq += 0.5 * u_dot_xi * u_dot_xi * 9.0;
            leq -= 0.5 * u_dot_u * 3.0;
            leq = leq * ln * c->w[q];
            pop[g + q * V] = leq;
        }
    }
}

static void s_outlet(const orc_simple *c, long V, double *pop, double *n, double *u, const int *walls) {
    const int D = c->dim, Q = c->Q;
    for (long g = 0; g < V; g++) {
        if (walls[g] != 3) continue;
        int p[3];
        s_pos(c, g, p);
        p[0] -= 1;
        const long src = s_index(c, p);
        n[g] = n[src];
        for (int d = 0; d < D; d++) u[g + d * V] = u[src + d * V];
        for (int q = 0; q < Q; q++) pop[g + q * V] = pop[src + q * V];
    }
}

static void s_collide(const orc_simple *c, long V, double *pop, double *u, const double *n, const double *psi,
                      const int *walls) {
    const int D = c->dim, Q = c->Q;
    const double om = c->omega;
    for (long g = 0; g < V; g++) {
        if (c->gravity ? walls[g] == 0 : walls[g] != 1) continue;
        int pos[3], np[3];
        s_pos(c, g, pos);
        double F[3] = {0., 0., 0.}, lu_post[3] = {0., 0., 0.};
        const double lpsi = psi[g];
        for (int a = 0; a < c->QE; a++) {
            for (int d = 0; d < D; d++) np[d] = ((pos[d] + c->e[d + a * D] + c->L[d]) % c->L[d]);
            const double npsi = psi[s_index(c, np)];
            for (int d = 0; d < D; d++) F[d] += c->e[d + a * D] * c->we[a] * npsi;
        }
        for (int d = 0; d < D; d++) F[d] *= -c->G * lpsi;
        if (c->gravity) F[1] += c->g;
        const double ln = n[g];
        double lu[3];
        if (c->forcing == 0) {
            for (int d = 0; d < D; d++) {
                lu[d] = u[g + V * d] + 0.5 * F[d] / ln;
                u[g + V * d] = lu[d];
            }
            double u_dot_u = 0., F_dot_u = 0.;
            for (int d = 0; d < D; d++) {
                u_dot_u += lu[d] * lu[d];
                F_dot_u += F[d] * lu[d];
            }
            for (int q = 0; q < Q; q++) {
                double u_dot_xi = 0., F_dot_xi = 0.;
                for (int d = 0; d < D; d++) {
                    u_dot_xi += lu[d] * c->xi[d + q * D];
                    F_dot_xi += F[d] * c->xi[d + q * D];
                }
                double leq = 1., lguo = 0.;
                leq += +u_dot_xi * 3.0 + 0.5 * u_dot_xi * u_dot_xi * 9.0;
                leq += -0.5 * u_dot_u * 3.0;
                leq = leq * ln * c->w[q];
                lguo += +F_dot_xi * 3.0 + F_dot_xi * u_dot_xi * 9.0;
                lguo += -F_dot_u * 3.0;
                lguo = lguo * c->w[q];
                pop[g + q * V] = pop[g + q * V] * (1. - om) + leq * om + (1. - 0.5 * om) * lguo;
            }
        } else {
            for (int d = 0; d < D; d++) lu[d] = u[g + V * d] + F[d] / ln / om;
            double u_dot_u = 0.;
            for (int d = 0; d < D; d++) u_dot_u += lu[d] * lu[d];
            for (int q = 0; q < Q; q++) {
                double u_dot_xi = 0.;
                for (int d = 0; d < D; d++) u_dot_xi += lu[d] * c->xi[d + q * D];
                double leq = 1.;
                leq += +u_dot_xi * 3.0 + 0.5 * u_dot_xi * u_dot_xi * 9.0;
                leq += -0.5 * u_dot_u * 3.0;
                leq = leq * ln * c->w[q];
                pop[g + q * V] = pop[g + q * V] * (1. - om) + leq * om;
                for (int d = 0; d < D; d++) lu_post[d] += pop[g + q * V] * c->xi[d + q * D];
            }
            for (int d = 0; d < D; d++) u[g + V * d] = 0.5 * (u[g + V * d] + lu_post[d] / ln);
        }
    }
}

static void s_moments_psi(const orc_simple *c, long V, const double *cur, double *n, double *u, double *psi,
                          const int *walls) {
    const int D = c->dim, Q = c->Q;
    for (long g = 0; g < V; g++) {  /* moments */
        if (walls[g] != 1) continue;
        double lu[3] = {0., 0., 0.}, ln = 0.;
        for (int q = 0; q < Q; q++) {
            const double lpop = cur[g + q * V];
            ln += lpop;
            for (int d = 0; d < D; d++) lu[d] += lpop * c->xi[d + q * D];
        }
        n[g] = ln;
        for (int d = 0; d < D; d++) u[g + d * V] = lu[d] / ln;
    }
    for (long g = 0; g < V; g++)  /* psi */
        if (walls[g]) psi[g] = psi_of(c->psi_kind, n[g]);
}

static void s_stream_bounce(const orc_simple *c, long V, const double *cur, double *nxt, const int *walls) {
    const int D = c->dim, Q = c->Q;
    for (long g = 0; g < V; g++) {  /* pull stream */
        int dp[3], sp[3];
        s_pos(c, g, dp);
        nxt[g] = cur[g];
        for (int q = 1; q < Q; q++) {
            for (int d = 0; d < D; d++) sp[d] = ((dp[d] - c->xi[d + q * D] + c->L[d]) % c->L[d]);
            nxt[g + q * V] = cur[s_index(c, sp) + q * V];
        }
    }
    for (long g = 0; g < V; g++) {  /* halfway bounce-back out of the walls */
        if (walls[g] != 0) continue;
        int sp[3], dp[3];
        s_pos(c, g, sp);
        nxt[g] = 0.;
        for (int q = 1; q < Q; q++) {
            const int qd = c->opposite[q];
            for (int d = 0; d < D; d++) dp[d] = ((sp[d] + c->xi[d + qd * D] + c->L[d]) % c->L[d]);
            nxt[s_index(c, dp) + qd * V] = nxt[g + q * V];
            nxt[g + q * V] = 0.;
        }
    }
}

int orc_simple_run(const orc_simple *c, double *pop_a, double *pop_b, double *n, double *u, double *psi,
                   const int *walls, int nsteps, int *swapped) {
    long V = 1;
    for (int d = 0; d < c->dim; d++) V *= c->L[d];
    double *cur = pop_a, *nxt = pop_b;
    for (int s = 0; s < nsteps; s++) {
        if (c->order == 1) {
            s_outlet(c, V, cur, n, u, walls);
            s_inlet(c, V, cur, n, u, walls);
            s_stream_bounce(c, V, cur, nxt, walls);
            double *t = cur; cur = nxt; nxt = t;
            s_moments_psi(c, V, cur, n, u, psi, walls);
            s_collide(c, V, cur, u, n, psi, walls);
            continue;
        }
        if (c->inout) {
            s_inlet(c, V, cur, n, u, walls);
            s_outlet(c, V, cur, n, u, walls);
        }
        s_moments_psi(c, V, cur, n, u, psi, walls);
        s_collide(c, V, cur, u, n, psi, walls);
        s_stream_bounce(c, V, cur, nxt, walls);
        double *t = cur; cur = nxt; nxt = t;
    }
    *swapped = (cur != pop_a);
    return 0;
}
