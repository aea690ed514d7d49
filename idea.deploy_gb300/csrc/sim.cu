// C ABI of the Shan-Chen step (include/sclbm.h): handle lifetime, device memory,
// the step loop (CUDA-graph replay of the two-pass step), read-back and the FP64
// reductions.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // CUcontext / CUresult types; the entry points come from the runtime
#include <cuda_runtime.h>

#include "../../include/sclbm.h"
#include "coeffs.h"
#include "launch.cuh"

using namespace sclbm;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

namespace sclbm {
// the last-error message of this thread, for the other translation units of
// the library (sclbm_last_error reads it)
int set_error(int code, const char *msg) {
    g_err = msg ? msg : "";
    return code;
}
void clear_error() { g_err.clear(); }
}  // namespace sclbm

namespace {

#define CUDA_TRY(call)                                                                                \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(SCLBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

constexpr int RED_THREADS = 256;
constexpr int GRAPH_STEPS = 32;  // steps per captured graph (even: buffers come back)

// ---- reductions (FP64 accumulation, per-block partials, host finishes) -----
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// reduce NV values per thread into out[blockIdx.x*NV + i]; op: 0 sum, 1 max
template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], const int (&op)[NV], double *out) {
    __shared__ double sh[NV][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        v[i] = op[i] ? warp_max(v[i]) : warp_sum(v[i]);
        if (lane == 0) sh[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) {
            double x = lane < RED_THREADS / 32 ? sh[i][lane] : (op[i] ? -INFINITY : 0.0);
            x = op[i] ? warp_max(x) : warp_sum(x);
            if (lane == 0) out[blockIdx.x * NV + i] = x;
        }
    }
}

// mass (sum of all f) and momentum sum_q xi_q f_q
template <class L, class Real>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_pop(const Real *__restrict__ pop, int64_t V, double rho0,
                                                           double *out) {
    constexpr int NV = 1 + L::D;
    double v[NV] = {};
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        double s = 0, j[L::D] = {};
#pragma unroll
        for (int q = 0; q < L::Q; q++) {
            const double f = (double)pop[(int64_t)q * V + g];
            s += f;
#pragma unroll
            for (int d = 0; d < L::D; d++)
                if (L::xi(q, d)) j[d] += L::xi(q, d) * f;
        }
        v[0] += s + rho0;  // sum_q w_q rho0 = rho0
#pragma unroll
        for (int d = 0; d < L::D; d++) v[1 + d] += j[d];
    }
    int op[NV] = {};
    block_reduce<NV>(v, op, out);
}

// add delta to the rest population (q = 0) of every cell
// Self-test of the bounded wait: an mbarrier that expects two arrivals gets
// one, so its phase never completes; the wait gives up after `polls` polls,
// records it in *err as the single-pass variants do, and the kernel returns.
// *err bit 1: the phase completed, which must not happen.
__global__ void k_bounded_wait_selftest(int *err, int polls) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 2);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive(&bar);
        bool dead = false;
        mbar_wait_bounded(&bar, 0, err, dead, polls);
        if (!dead) atomicOr(err, 2);
    }
}

template <class Real>
__global__ void __launch_bounds__(RED_THREADS) k_add_rest(Real *__restrict__ pop0, int64_t V, Real delta) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x)
        pop0[g] += delta;
}

// CheckUConvergenceSCMP: sum_d |u - u_old| summed, max |u|^2; then u_old = u
template <class Real>
__global__ void __launch_bounds__(RED_THREADS) k_check_u(const Real *__restrict__ u, Real *__restrict__ u_old,
                                                        int D, int64_t V, double *out) {
    double v[2] = {0.0, 0.0};
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        double dsum = 0, n2 = 0;
        for (int d = 0; d < D; d++) {
            const double a = (double)u[(int64_t)d * V + g];
            const double b = (double)u_old[(int64_t)d * V + g];
            n2 += a * a;
            dsum += fabs(a - b);
            u_old[(int64_t)d * V + g] = u[(int64_t)d * V + g];
        }
        v[0] += dsum;
        v[1] = fmax(v[1], n2);
    }
    int op[2] = {0, 1};
    block_reduce<2>(v, op, out);
}

// mass and first moments of the density (centre of mass)
template <class Real>
__global__ void __launch_bounds__(RED_THREADS) k_com(const Real *__restrict__ dn, double rho0, int D, int L0, int L1,
                                                    int64_t V, double *out) {
    double v[4] = {0, 0, 0, 0};
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const double n = rho0 + (double)dn[g];
        const int x = (int)(g % L0);
        const int y = (int)((g / L0) % L1);
        const int z = (int)(g / ((int64_t)L0 * L1));
        v[0] += n;
        v[1] += n * x;
        v[2] += n * y;
        v[3] += D == 3 ? n * z : 0.0;
    }
    int op[4] = {0, 0, 0, 0};
    block_reduce<4>(v, op, out);
}

template <class Real>
__global__ void __launch_bounds__(RED_THREADS) k_finite(const Real *__restrict__ dn, double rho0, int64_t V,
                                                       double *out) {
    double v[2] = {0.0, 0.0};
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        const double n = rho0 + (double)dn[g];
        if (!isfinite(n)) v[0] = 1.0;
        else v[1] = fmax(v[1], fabs(n));
    }
    int op[2] = {1, 1};
    block_reduce<2>(v, op, out);
}

// ---- initial profiles (idpy/LBM/MultiPhaseKernels.py:44-112,605-777) -----
enum { PROF_RADIAL = 0, PROF_FLAT = 1, PROF_SINGLE_FLAT = 2, PROF_CYLINDER = 3 };

template <class Real>
__global__ void k_profile(Real *__restrict__ dn, Real *__restrict__ u, int kind, int D, int L0, int L1, int L2,
                          int64_t V, double n_g, double n_l, double R, double width, int dir, int full, double rho0) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < V; g += (int64_t)gridDim.x * blockDim.x) {
        int pos[3];
        pos[0] = (int)(g % L0);
        pos[1] = (int)((g / L0) % L1);
        pos[2] = D == 3 ? (int)(g / ((int64_t)L0 * L1)) : 0;
        const int Ls[3] = {L0, L1, L2};
        const double dnv = full ? (n_l - n_g) : (n_g - n_l);
        double n = 0;
        if (kind == PROF_RADIAL || kind == PROF_CYLINDER) {
            int r2 = 0;
            for (int d = 0; d < D; d++) {
                if (kind == PROF_CYLINDER && d == dir) continue;
                const int t = Ls[d] / 2 - pos[d];
                r2 += t * t;
            }
            const double r = sqrt((double)r2);
            n = 0.5 * (n_g + n_l) - 0.5 * dnv * tanh(r - R);
        } else if (kind == PROF_FLAT) {
            const int L = Ls[dir], x = pos[dir], x0 = L / 2, xm = L / 2;
            int xp;
            if (x0 - xm >= 0) xp = (x < x0 - xm) ? x - (x0 - xm) + L : x - (x0 - xm);
            else xp = (x < x0 + xm) ? x - (x0 + xm) + L : x - (x0 + xm);
            const double prof = tanh((double)xp - (xm - 0.5 * width)) - tanh((double)xp - (xm + 0.5 * width));
            n = 0.5 * (n_g + n_l) + 0.5 * dnv * (prof - 1.0);
        } else {
            const int x0 = Ls[dir] / 2;
            n = n_g + dnv * ((tanh((double)(pos[dir] - x0)) + 1.0) * 0.5);
        }
        dn[g] = (Real)(n - rho0);
        for (int d = 0; d < D; d++) u[(int64_t)d * V + g] = Real(0);
    }
}

}  // namespace

// ============================================================================
struct sclbm_sim {
    int device = 0;
    cudaStream_t st = nullptr;
    int D = 0, Q = 0, QE = 0, K = 0, order = 0;
    int L[3] = {1, 1, 1};
    int64_t V = 0;
    bool fp32 = false, mrt = false;
    size_t rs = 8;
    double rho0 = 0, c2 = 1.0 / 3, G = 0;
    std::vector<double> w, we;
    std::vector<int> xi, e;
    int psi_kind = 0, literals = 0, sms = 1;
    const KernelOps *ops = nullptr;
    std::vector<unsigned char> sp, ep;  // launch parameter blocks
    void *pop[2] = {nullptr, nullptr};
    int cur = 0;
    void *dn = nullptr, *psi = nullptr, *u = nullptr, *u_old = nullptr;
    unsigned char *walls = nullptr;  // GetWalls: 1 fluid, 0 wall (null: no walls)
    void *psi_w = nullptr;           // the psi the walls keep
    // fluctuations (sclbm_set_fluctuations): generator kind (0: off), one or two
    // generators per random moment, their states on the device, the noise operator
    int noise_kind = 0, noise_indep = 0, noise_streams = 0;
    bool noise_sparse = false;      // the operator fits the single-pass kernel's nonzero pattern
    void *seeds = nullptr;
    std::vector<double> noise_m2var, noise_coef;
    std::vector<unsigned char> np;  // noise launch parameter block
    int ngrid = 0;                  // noise kernel grid (resident CTAs, capped by the cells)
    double tau_bgk = 1.0;           // BGK relaxation time of the current operator
    // the "simple" step family (sclbm_set_simple): 0 off, SCLBM_SIMPLE_GUO / _SC
    int simple_mode = 0, simple_inout = 0, simple_walls = 0;
    bool sym_weights = true;  // opposite directions / stencil vectors carry equal weights
    SimpleParams spar = {};
    double *red = nullptr;
    int red_blocks = 0;
    int dgrid = 0, fgrid = 0, ugrid = 0;
    FusedGeom fg = {};
    int fused_grid = 0, path = SCLBM_PATH_AUTO, chunk_override = 0;
    int staging = -1;  // requested SCLBM_STAGE_* flags of the 3D single pass (-1: automatic)
    int tile = -1;     // requested tile shape (index into kTiles) of the 3D paired single pass (-1: automatic)
    int item_order = -1;  // requested order of the single pass's work items (-1: automatic, 0)
    // tensor maps of the two population buffers (4D: x, y, plane, q; box of one
    // tile plane), encoded when a staged variant with TMA loads is planned
    CUtensorMap tmap[2];
    bool tmap_ok = false;
    int *flag_host = nullptr, *flag_dev = nullptr;  // set by a device wait that gave up (mapped pinned int)
    bool n_set = false, u_set = false, pop_set = false, moments_fresh = false;
    bool dn_fresh = true;  // dn holds the density of the current populations
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int64_t device_bytes = 0;
    void *stage = nullptr;  // pinned host staging buffer (lazy)
    int transfer = SCLBM_TRANSFER_AUTO;
    bool pageable_access = false;  // the device reads and writes pageable host memory (coherent C2C)
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
};

namespace {

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int alloc(sclbm_sim *s, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(SCLBM_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    }
    s->device_bytes += (int64_t)bytes;
    return SCLBM_OK;
}

void release(sclbm_sim *s) {
    for (auto &g : s->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    for (void *p : {s->pop[0], s->pop[1], s->dn, s->psi, s->u, s->u_old, (void *)s->red, (void *)s->walls, s->psi_w,
                    s->seeds})
        if (p) cudaFree(p);
    for (auto &ev : s->stage_ev)
        if (ev) cudaEventDestroy(ev), ev = nullptr;
    if (s->stage) cudaFreeHost(s->stage);
    if (s->flag_host) cudaFreeHost(s->flag_host);
    if (s->st) cudaStreamDestroy(s->st);
}

const int *compiled_xi(int D, int q) {
    static int t2[9 * 2], t3[19 * 3];
    static bool init = false;
    if (!init) {
        for (int i = 0; i < 9; i++)
            for (int d = 0; d < 2; d++) t2[i * 2 + d] = D2Q9::xi(i, d);
        for (int i = 0; i < 19; i++)
            for (int d = 0; d < 3; d++) t3[i * 3 + d] = D3Q19::xi(i, d);
        init = true;
    }
    if (D == 2 && q == 9) return t2;
    if (D == 3 && q == 19) return t3;
    return nullptr;
}

template <class S>
bool stencil_is(const int *e, int qe) {
    if (qe != S::QE) return false;
    for (int a = 0; a < qe; a++)
        for (int d = 0; d < S::D; d++)
            if (e[a * S::D + d] != S::e(a, d)) return false;
    return true;
}

int stencil_order(int D, const int *e, int qe) {
    if (D == 2) {
        if (stencil_is<D2E4>(e, qe)) return 4;
        if (stencil_is<D2E6>(e, qe)) return 6;
        if (stencil_is<D2E8>(e, qe)) return 8;
    } else {
        if (stencil_is<D3E4>(e, qe)) return 4;
        if (stencil_is<D3E6>(e, qe)) return 6;
        if (stencil_is<D3E8>(e, qe)) return 8;
    }
    return 0;
}

// the single-pass kernels pair every lattice direction and force-stencil vector
// with its opposite and assume equal weights for the two (true of the D2Q9 /
// D3Q19 lattices and the isotropic E4-E8 stencils)
bool weights_symmetric(const sclbm_params *p) {
    auto sym = [&](const int *v, const double *w, int n) {
        for (int a = 0; a < n; a++) {
            int b = -1;
            for (int k = 0; k < n && b < 0; k++) {
                bool opp = true;
                for (int d = 0; d < p->dim; d++) opp = opp && v[k * p->dim + d] == -v[a * p->dim + d];
                if (opp) b = k;
            }
            if (b < 0 || w[a] != w[b]) return false;
        }
        return true;
    };
    return sym(p->xi, p->w, p->q) && sym(p->e, p->we, p->qe);
}

// the single-pass kernel indexes populations with 32-bit offsets (q*V + cell)
bool fused_fits(const sclbm_sim *s) { return (int64_t)s->Q * s->V < ((int64_t)1 << 31); }

bool fused_path(const sclbm_sim *s) {
    return s->ops->fused != nullptr && s->path != SCLBM_PATH_TWO_PASS && fused_fits(s) && s->sym_weights &&
           (!s->walls || s->ops->fused_walls != nullptr) && !s->simple_mode &&
           (!s->noise_kind || (s->ops->fused_noise != nullptr && !s->noise_indep && s->noise_sparse &&
                               (int64_t)s->noise_streams * s->V < ((int64_t)1 << 31)));
}

// density + psi of the current populations (fluid cells only with walls)
cudaError_t density_pass(sclbm_sim *s) {
    if (s->walls)
        return s->ops->density_walls(s->pop[s->cur], s->dn, s->psi, s->walls, s->psi_w, s->sp.data(), s->dgrid, s->st);
    return s->ops->density(s->pop[s->cur], s->dn, s->psi, s->sp.data(), s->dgrid, s->st);
}

// the SC inlet/outlet loop streams before it collides (MultiPhase.py:735-887)
bool simple_stream_first(const sclbm_sim *s) { return s->simple_mode == SCLBM_SIMPLE_SC && s->simple_inout; }

int simple_kernels(const sclbm_sim *s) {
    if (simple_stream_first(s)) return 5;
    return (s->simple_inout ? 2 : 0) + 2;
}

// one step of the simple family; ev (optional) gets an event after each kernel
int launch_simple(sclbm_sim *s, cudaEvent_t *ev) {
    const KernelOps *o = s->ops;
    const SimpleParams &p = s->spar;
    const int sc = s->simple_mode == SCLBM_SIMPLE_SC;
    const unsigned char *walls = s->simple_walls ? s->walls : nullptr;
    void *cur = s->pop[s->cur], *nxt = s->pop[s->cur ^ 1];
    int k = 0;
    cudaError_t e = cudaSuccess;
    auto mark = [&]() {
        if (ev && e == cudaSuccess) e = cudaEventRecord(ev[k], s->st);
        k++;
    };
    if (simple_stream_first(s)) {
        e = o->simple_outlet(cur, s->dn, s->u, walls, p, s->dgrid, s->st);
        mark();
        if (e == cudaSuccess) e = o->simple_inlet(cur, s->dn, s->u, walls, p, s->dgrid, s->st);
        mark();
        if (e == cudaSuccess) e = o->simple_stream(cur, nxt, walls, p, s->fgrid, s->st);
        mark();
        if (e == cudaSuccess) e = o->simple_moments(nxt, s->dn, s->u, s->psi, walls, p, s->dgrid, s->st);
        mark();
        if (e == cudaSuccess) e = o->simple_collide(sc, 0, nxt, nxt, s->dn, s->u, s->psi, walls, p, s->fgrid, s->st);
        mark();
    } else {
        if (s->simple_inout) {
            e = o->simple_inlet(cur, s->dn, s->u, walls, p, s->dgrid, s->st);
            mark();
            if (e == cudaSuccess) e = o->simple_outlet(cur, s->dn, s->u, walls, p, s->dgrid, s->st);
            mark();
        }
        if (e == cudaSuccess) e = o->simple_moments(cur, s->dn, s->u, s->psi, walls, p, s->dgrid, s->st);
        mark();
        if (e == cudaSuccess) e = o->simple_collide(sc, 1, cur, nxt, s->dn, s->u, s->psi, walls, p, s->fgrid, s->st);
        mark();
    }
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    s->cur ^= 1;
    return SCLBM_OK;
}

// enqueue the kernels of one step; ev (optional) gets an event after each kernel
int launch_step(sclbm_sim *s, cudaEvent_t *ev = nullptr) {
    const KernelOps *o = s->ops;
    cudaError_t e;
    if (s->simple_mode) return launch_simple(s, ev);
    if (fused_path(s)) {
        if (s->walls)
            e = o->fused_walls(s->pop[s->cur], s->pop[s->cur ^ 1], s->sp.data(), s->fg, s->walls, s->psi_w,
                               s->fused_grid, s->st);
        else if (s->noise_kind)
            e = o->fused_noise(s->pop[s->cur], s->pop[s->cur ^ 1], s->sp.data(), s->fg, s->seeds, s->np.data(),
                               s->fused_grid, s->st);
        else
            e = o->fused(s->pop[s->cur], s->pop[s->cur ^ 1], s->sp.data(), s->fg, s->fused_grid,
                         (s->fg.stg & STG_OWN_TMA) ? (const void *)&s->tmap[s->cur] : nullptr, s->st);
        if (ev && e == cudaSuccess) e = cudaEventRecord(ev[0], s->st);
    } else {
        e = density_pass(s);
        if (ev && e == cudaSuccess) e = cudaEventRecord(ev[0], s->st);
        if (e == cudaSuccess && s->noise_kind)
            e = o->fcs_noise(s->pop[s->cur], s->pop[s->cur ^ 1], s->dn, s->psi, s->seeds, s->sp.data(), s->np.data(),
                             s->ngrid, s->st);
        else if (e == cudaSuccess && s->walls)
            e = o->fcs_walls(s->pop[s->cur], s->pop[s->cur ^ 1], s->dn, s->psi, s->walls, s->sp.data(), s->fgrid,
                             s->st);
        else if (e == cudaSuccess)
            e = o->fcs(s->pop[s->cur], s->pop[s->cur ^ 1], s->dn, s->psi, s->sp.data(), s->fgrid, s->st);
        if (ev && e == cudaSuccess) e = cudaEventRecord(ev[1], s->st);
    }
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    s->cur ^= 1;
    return SCLBM_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// to the driver library)
using PfnEncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
PfnEncodeTiled encode_tiled() {
    static PfnEncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PfnEncodeTiled>(f);
        cudaGetLastError();
    });
    return fn;
}

// the population buffers as 4D FP32 tensors (x, y, plane, q) with a box of one
// tile plane (TX, TY, 1, Q); TMA needs 16-byte strides, so Lx % 4 == 0
bool encode_tmaps(sclbm_sim *s) {
    const KernelOps *o = s->ops;
    if (s->D != 3 || s->L[0] % 4 != 0) return false;
    PfnEncodeTiled enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)s->L[0], (cuuint64_t)s->L[1], (cuuint64_t)s->L[2], (cuuint64_t)s->Q};
    const cuuint64_t strides[3] = {(cuuint64_t)s->L[0] * 4, (cuuint64_t)s->L[0] * s->L[1] * 4, (cuuint64_t)s->V * 4};
    const cuuint32_t box[4] = {(cuuint32_t)o->fused_tx, (cuuint32_t)o->fused_ty, 1, (cuuint32_t)s->Q};
    const cuuint32_t unit[4] = {1, 1, 1, 1};
    for (int b = 0; b < 2; b++) {
        if (enc(&s->tmap[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, s->pop[b], dims, strides, box, unit,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

// staging of the 3D single pass: the requested flags where the kernel set has
// them and the box supports them; automatic (-1): none until measured
int plan_staging(sclbm_sim *s, bool pairs) {
    if (!pairs || s->walls || s->noise_kind || s->staging <= 0) return 0;
    int stg = s->staging & s->ops->fused_stg_mask;
    if (stg & STG_OWN_TMA) {
        if (!s->tmap_ok) s->tmap_ok = encode_tmaps(s);
        if (!s->tmap_ok) stg &= ~STG_OWN_TMA;
    }
    return stg;
}

// ---- tuned configurations, cached per (lattice, stencil, operator, box, device) ----
// the kernel set (lattice, stencil, operator kind, precision, arithmetic) is
// identified by its KernelOps table; walls, box and SM count complete the key
struct TuneKey {
    const KernelOps *ops;
    int v[6];
    bool operator<(const TuneKey &o) const {
        if (ops != o.ops) return std::less<const KernelOps *>()(ops, o.ops);
        return std::lexicographical_compare(v, v + 6, o.v, o.v + 6);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, sclbm_tuning> g_tune_cache;

TuneKey tune_key(const sclbm_sim *s) {
    return TuneKey{s->ops, {s->walls ? 1 : 0, s->noise_kind, s->L[0], s->L[1], s->L[2], s->sms}};
}

bool cached_tuning(const sclbm_sim *s, sclbm_tuning *t) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(tune_key(s));
    if (it == g_tune_cache.end()) return false;
    *t = it->second;
    return true;
}

// work decomposition of the single-pass kernel: tiles of the leading
// dimensions x chunks of the marching dimension, sized so the items fill the
// resident CTAs in whole waves with a small halo-plane overhead per chunk.
// A handle left on the automatic choice (path AUTO, no chunk, staging -1)
// takes the configuration sclbm_autotune found for its key, if any.
void plan_fused(sclbm_sim *s) {
    const KernelOps *o = s->ops;
    if (!o->fused) return;
    sclbm_tuning tuned;
    if (s->path == SCLBM_PATH_AUTO && s->chunk_override == 0 && s->staging < 0 && cached_tuning(s, &tuned)) {
        const int saved_path = s->path, saved_chunk = s->chunk_override, saved_stg = s->staging, saved_tile = s->tile,
                  saved_order = s->item_order;
        s->path = tuned.path == SCLBM_PATH_FUSED ? SCLBM_PATH_FUSED : SCLBM_PATH_AUTO;
        s->chunk_override = tuned.chunk;
        s->staging = tuned.staging;
        s->tile = tuned.tile;
        s->item_order = tuned.order;
        plan_fused(s);
        s->path = saved_path;
        s->chunk_override = saved_chunk;
        s->staging = saved_stg;
        s->tile = saved_tile;
        s->item_order = saved_order;
        return;
    }
    FusedGeom &g = s->fg;
    for (int d = 0; d < 3; d++) g.L[d] = d < s->D ? s->L[d] : 1;
    g.V = s->V;
    g.tiles_x = (s->L[0] + o->fused_tx - 1) / o->fused_tx;
    g.tiles_y = s->D == 3 ? (s->L[1] + o->fused_ty - 1) / o->fused_ty : 1;
    const int Lm = s->D == 3 ? s->L[2] : s->L[1];
    // paired halo loads where they apply (the automatic choice: 12-14% faster
    // than one cell per load at 256^3 D3Q19 E6/E8, bit-identical results)
    g.pairs = (s->path == SCLBM_PATH_FUSED_PAIRS || s->path == SCLBM_PATH_AUTO) && s->D == 3 && s->L[0] % 2 == 0 &&
              o->fused_r % 2 == 0;
    g.stg = plan_staging(s, g.pairs);
    g.err = s->flag_dev;
    // another tile shape (3D paired BGK, not staged, no walls or noise)
    g.tile = 0;
    if (g.pairs && !g.stg && !s->walls && !s->noise_kind && s->tile > 0 && s->tile < N_TILES &&
        (o->fused_tile_mask >> s->tile & 1))
        g.tile = s->tile;
    if (g.tile) {
        g.tiles_x = (s->L[0] + kTiles[g.tile].tx - 1) / kTiles[g.tile].tx;
        g.tiles_y = (s->L[1] + kTiles[g.tile].ty - 1) / kTiles[g.tile].ty;
    }
    // work-item order (k_fused only; y fastest exists in 3D only)
    g.order = (s->item_order > 0 && s->item_order <= (s->D == 3 ? 2 : 1) && !s->walls && !s->noise_kind && !g.stg)
                  ? s->item_order
                  : 0;
    const int resident = s->sms * (s->noise_kind ? o->fused_noise_occupancy(s->noise_kind)
                                   : s->walls    ? o->fused_walls_occupancy()
                                                 : o->fused_occupancy(g.pairs, g.stg, g.tile));
    const int base = g.tiles_x * g.tiles_y;
    int best_c = 1;
    double best = -1;
    for (int c = 1; c <= std::max(1, Lm / (2 * o->fused_r + 2)); c++) {
        const int chunk = (Lm + c - 1) / c;
        const int items = base * ((Lm + chunk - 1) / chunk);
        const int waves = (items + resident - 1) / resident;
        const double fill = (double)items / ((double)waves * resident);
        const double halo = (double)chunk / (chunk + 2.0 * o->fused_r);
        const double eff = fill * halo;  // resident-slot fill x share of planes that are not preamble
        if (eff > best + 1e-9) {
            best = eff;
            best_c = c;
        }
    }
    g.chunk = s->chunk_override > 0 ? std::min(s->chunk_override, Lm) : (Lm + best_c - 1) / best_c;
    g.chunks = (Lm + g.chunk - 1) / g.chunk;
    g.items = base * g.chunks;
    s->fused_grid = std::max(1, std::min(g.items, resident));
}

int build_graph(sclbm_sim *s, int parity) {
    const int saved = s->cur;
    s->cur = parity;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    int rc = SCLBM_OK;
    for (int i = 0; i < GRAPH_STEPS && rc == SCLBM_OK; i++) rc = launch_step(s);
    cudaError_t ce = cudaStreamEndCapture(s->st, &g);
    s->cur = saved;
    if (rc != SCLBM_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess) return fail(SCLBM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&s->graph[parity], g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fail(SCLBM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    return SCLBM_OK;
}

int run_steps(sclbm_sim *s, int64_t n) {
    while (n >= GRAPH_STEPS) {
        if (!s->graph[s->cur]) {
            int rc = build_graph(s, s->cur);
            if (rc) return rc;
        }
        CUDA_TRY(cudaGraphLaunch(s->graph[s->cur], s->st));
        n -= GRAPH_STEPS;  // even number of steps: s->cur unchanged
    }
    for (int64_t i = 0; i < n; i++) {
        int rc = launch_step(s);
        if (rc) return rc;
    }
    return SCLBM_OK;
}

// Host <-> device transfers go through a pinned staging buffer in two halves
// (double-buffered: the copy of one chunk overlaps the conversion of the
// other).  Device arrays hold Real (FP64, or FP32 deviations); host arrays are
// FP64 values, minus / plus an optional per-plane shift (w_q rho0, rho0).
constexpr size_t STAGE_BYTES = size_t(32) << 20;

int ensure_stage(sclbm_sim *s) {
    if (s->stage) return SCLBM_OK;
    cudaError_t e = cudaMallocHost(&s->stage, STAGE_BYTES);
    if (e != cudaSuccess) {
        s->stage = nullptr;
        cudaGetLastError();
        return fail(SCLBM_ERR_NOMEM, "pinned staging buffer: %s", cudaGetErrorString(e));
    }
    for (auto &ev : s->stage_ev) {
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "staging event: %s", cudaGetErrorString(e));
    }
    return SCLBM_OK;
}

inline double shift_at(const double *plane_shift, int64_t i, int64_t plane) {
    return plane_shift ? plane_shift[i / plane] : 0.0;
}

// Direct transfers: a kernel reads or writes the caller's FP64 host array itself
// (over NVLink-C2C on Grace-Blackwell) and converts on the fly, with the same
// per-element arithmetic as the staged path (x - shift rounded once to Real;
// (double)x + shift), so both give identical arrays.  Used when the host
// array is pinned / registered memory, or when the device reports access to
// pageable host memory; otherwise the staged path runs.
struct ShiftTab {
    double v[27];
    int64_t plane;
};

template <class Real>
__global__ void __launch_bounds__(256) k_from_host(Real *__restrict__ dst, const double *__restrict__ src, int64_t count,
                                                   const ShiftTab sh) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (Real)(src[i] - sh.v[i / sh.plane]);
}

template <class Real>
__global__ void __launch_bounds__(256) k_to_host(double *__restrict__ dst, const Real *__restrict__ src, int64_t count,
                                                 const ShiftTab sh) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i] + sh.v[i / sh.plane];
}

// device-usable address of a host array for the direct path, or null
const void *direct_address(sclbm_sim *s, const void *host, int64_t count, int64_t plane) {
    if (s->transfer == SCLBM_TRANSFER_STAGED || plane <= 0 || (count + plane - 1) / plane > 27) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost)
        return a.devicePointer ? a.devicePointer : host;
    cudaGetLastError();
    return s->pageable_access ? host : nullptr;
}

bool fill_shift(ShiftTab &sh, const double *plane_shift, int64_t count, int64_t plane) {
    sh.plane = plane;
    const int64_t np = (count + plane - 1) / plane;
    for (int64_t k = 0; k < 27; k++) sh.v[k] = (plane_shift && k < np) ? plane_shift[k] : 0.0;
    return true;
}

int d2h_real(sclbm_sim *s, const void *src, double *dst, int64_t count, const double *plane_shift, int64_t plane) {
    if (count <= 0) return SCLBM_OK;
    if (void *d = (void *)direct_address(s, dst, count, plane)) {
        ShiftTab sh;
        fill_shift(sh, plane_shift, count, plane);
        const int grid = s->sms * 8;
        if (s->fp32) k_to_host<float><<<grid, 256, 0, s->st>>>((double *)d, (const float *)src, count, sh);
        else k_to_host<double><<<grid, 256, 0, s->st>>>((double *)d, (const double *)src, count, sh);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(s->st));
        return SCLBM_OK;
    }
    if (s->transfer == SCLBM_TRANSFER_DIRECT) return fail(SCLBM_ERR_UNSUPPORTED, "host array not device-accessible");
    int rc = ensure_stage(s);
    if (rc) return rc;
    const int64_t per = (int64_t)(STAGE_BYTES / 2 / s->rs);
    const int64_t nchunk = (count + per - 1) / per;
    char *half[2] = {(char *)s->stage, (char *)s->stage + STAGE_BYTES / 2};
    auto issue = [&](int64_t c) -> cudaError_t {
        const int64_t off = c * per, len = std::min(per, count - off);
        cudaError_t e = cudaMemcpyAsync(half[c & 1], (const char *)src + off * s->rs, len * s->rs,
                                        cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess) e = cudaEventRecord(s->stage_ev[c & 1], s->st);
        return e;
    };
    if (nchunk > 0) CUDA_TRY(issue(0));
    for (int64_t c = 0; c < nchunk; c++) {
        CUDA_TRY(cudaEventSynchronize(s->stage_ev[c & 1]));
        if (c + 1 < nchunk) CUDA_TRY(issue(c + 1));
        const int64_t off = c * per, len = std::min(per, count - off);
        if (s->fp32) {
            const float *h = (const float *)half[c & 1];
            for (int64_t i = 0; i < len; i++) dst[off + i] = (double)h[i] + shift_at(plane_shift, off + i, plane);
        } else {
            const double *h = (const double *)half[c & 1];
            for (int64_t i = 0; i < len; i++) dst[off + i] = h[i] + shift_at(plane_shift, off + i, plane);
        }
    }
    return SCLBM_OK;
}

int h2d_real(sclbm_sim *s, void *dst, const double *src, int64_t count, const double *plane_shift, int64_t plane) {
    if (count <= 0) return SCLBM_OK;
    if (const void *d = direct_address(s, src, count, plane)) {
        ShiftTab sh;
        fill_shift(sh, plane_shift, count, plane);
        const int grid = s->sms * 8;
        if (s->fp32) k_from_host<float><<<grid, 256, 0, s->st>>>((float *)dst, (const double *)d, count, sh);
        else k_from_host<double><<<grid, 256, 0, s->st>>>((double *)dst, (const double *)d, count, sh);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(s->st));
        return SCLBM_OK;
    }
    if (s->transfer == SCLBM_TRANSFER_DIRECT) return fail(SCLBM_ERR_UNSUPPORTED, "host array not device-accessible");
    int rc = ensure_stage(s);
    if (rc) return rc;
    const int64_t per = (int64_t)(STAGE_BYTES / 2 / s->rs);
    const int64_t nchunk = (count + per - 1) / per;
    char *half[2] = {(char *)s->stage, (char *)s->stage + STAGE_BYTES / 2};
    for (int64_t c = 0; c < nchunk; c++) {
        if (c >= 2) CUDA_TRY(cudaEventSynchronize(s->stage_ev[c & 1]));  // half free again
        const int64_t off = c * per, len = std::min(per, count - off);
        if (s->fp32) {
            float *h = (float *)half[c & 1];
            for (int64_t i = 0; i < len; i++) h[i] = (float)(src[off + i] - shift_at(plane_shift, off + i, plane));
        } else {
            double *h = (double *)half[c & 1];
            for (int64_t i = 0; i < len; i++) h[i] = src[off + i] - shift_at(plane_shift, off + i, plane);
        }
        CUDA_TRY(cudaMemcpyAsync((char *)dst + off * s->rs, half[c & 1], len * s->rs, cudaMemcpyHostToDevice,
                                 s->st));
        CUDA_TRY(cudaEventRecord(s->stage_ev[c & 1], s->st));
    }
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return SCLBM_OK;
}

int finish_partials(sclbm_sim *s, int nv, std::vector<double> &part) {
    part.resize((size_t)s->red_blocks * nv);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(part.data(), s->red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return SCLBM_OK;
}

int init_pop(sclbm_sim *s) {
    cudaError_t e = s->ops->init_pop(s->pop[s->cur], s->dn, s->u, s->ep.data(), s->fgrid, s->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "init populations: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    s->pop_set = true;
    s->moments_fresh = false;
    return SCLBM_OK;
}

int profile(sclbm_sim *s, int kind, double n_g, double n_l, double R, double width, int dir, int full) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (dir < 0 || dir >= s->D) return fail(SCLBM_ERR_ARG, "direction %d out of range", dir);
    DevGuard dg(s->device);
    if (s->fp32)
        k_profile<float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((float *)s->dn, (float *)s->u, kind, s->D, s->L[0],
                                                                   s->L[1], s->L[2], s->V, n_g, n_l, R, width, dir,
                                                                   full, s->rho0);
    else
        k_profile<double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((double *)s->dn, (double *)s->u, kind, s->D,
                                                                    s->L[0], s->L[1], s->L[2], s->V, n_g, n_l, R,
                                                                    width, dir, full, s->rho0);
    CUDA_TRY(cudaGetLastError());
    s->n_set = s->u_set = true;
    return init_pop(s);
}


// build the collision operator and launch parameters; pick the kernel set
int configure(sclbm_sim *s, int collision, double tau, const double *mrt_s, const double *coll_a,
              const double *coll_b) {
    if (collision != SCLBM_COLL_BGK && collision != SCLBM_COLL_MRT)
        return fail(SCLBM_ERR_ARG, "collision %d", collision);
    if ((coll_a == nullptr) != (coll_b == nullptr)) return fail(SCLBM_ERR_ARG, "coll_a and coll_b go together");
    if (collision == SCLBM_COLL_BGK && !coll_a && !(tau > 0)) return fail(SCLBM_ERR_ARG, "tau must be > 0");
    if (collision == SCLBM_COLL_MRT && !coll_a && !mrt_s)
        return fail(SCLBM_ERR_ARG, "MRT needs the relaxation matrix mrt_s");
    // MRT whose relaxation matrix is s*I is exactly BGK with omega = s (the
    // equilibrium part M^-1 S M, the relaxation M^-1 (I-S) M and the Guo part
    // Mn^-1 (I - S/2) Mn all reduce to multiples of I): the fused-arithmetic
    // paths run the sparse BGK kernels for it; the reference-arithmetic path
    // keeps the reference's expanded MRT expression.
    double uniform_rate = 0;
    if (collision == SCLBM_COLL_MRT && !coll_a && mrt_s && !(!s->fp32 && s->literals == SCLBM_LIT_ROUND15)) {
        bool uni = mrt_s[0] > 0;
        for (int i = 0; i < s->Q && uni; i++)
            for (int j = 0; j < s->Q && uni; j++) uni = mrt_s[(size_t)i * s->Q + j] == (i == j ? mrt_s[0] : 0.0);
        if (uni) {
            uniform_rate = mrt_s[0];
            collision = SCLBM_COLL_BGK;
        }
    }
    CollisionSpec cs;
    cs.dim = s->D;
    cs.q = s->Q;
    cs.xi = s->xi.data();
    cs.w = s->w.data();
    cs.c2 = s->c2;
    cs.collision = coll_a ? SCLBM_COLL_BGK : collision;  // equilibrium table always built
    cs.tau = coll_a ? 1.0 : tau;
    cs.omega = coll_a ? 0.0 : uniform_rate;
    cs.mrt_s = mrt_s;
    cs.literals = s->fp32 ? SCLBM_LIT_EXACT : s->literals;
    CollisionTables t;
    std::string err;
    if (build_collision(cs, t, err)) return fail(SCLBM_ERR_UNSUPPORTED, "collision operator: %s", err.c_str());
    if (coll_a) {
        t.A.assign(coll_a, coll_a + (size_t)s->Q * s->Q);
        t.B.assign(coll_b, coll_b + (size_t)s->Q * t.K);
    }
    const bool mrt = collision == SCLBM_COLL_MRT || coll_a != nullptr;
    // FP64 with the reference's literals also uses the reference's arithmetic
    const bool strict = !s->fp32 && s->literals == SCLBM_LIT_ROUND15;
    const KernelOps *ops = select_ops(s->D, s->order, mrt, s->fp32, strict);
    if (!ops) return fail(SCLBM_ERR_UNSUPPORTED, "no kernels for this configuration");
    if (s->noise_kind && !ops->fcs_noise)
        return fail(SCLBM_ERR_UNSUPPORTED, "the fluctuating step is BGK only (switch the fluctuations off first)");
    if (s->simple_mode && mrt)
        return fail(SCLBM_ERR_UNSUPPORTED, "the simple step family is BGK (switch it off first)");
    bool a_nonzero = false;
    for (int q = 0; q < s->Q; q++) a_nonzero = a_nonzero || t.A[(size_t)q * s->Q + q] != 0.0;
    HostSetup h;
    for (int d = 0; d < 3; d++) h.L[d] = d < s->D ? s->L[d] : 1;
    h.V = s->V;
    h.rho0 = s->rho0;
    h.G = s->G;
    h.psi_kind = s->psi_kind;
    h.we = s->we.data();
    h.A = t.A.data();
    h.B = t.B.data();
    h.Beq = t.Beq.data();
    h.a_nonzero = a_nonzero;
    h.omega = (!mrt && !coll_a) ? (uniform_rate > 0 ? uniform_rate : 1.0 / tau) : 0.0;
    h.w = s->w.data();
    // lattice weights symmetric under xi -> -xi and c2 = 1/3: what the factored form assumes
    bool sym = std::fabs(s->c2 - 1.0 / 3.0) < 1e-12;
    for (int q = 0; q < s->Q && sym; q++)
        for (int k = 0; k < s->Q; k++) {
            bool opp = true;
            for (int d = 0; d < s->D; d++) opp = opp && s->xi[(size_t)q * s->D + d] == -s->xi[(size_t)k * s->D + d];
            if (opp) sym = sym && s->w[q] == s->w[k];
        }
    h.factored = !s->fp32 && !mrt && h.omega > 0 && sym && s->literals == SCLBM_LIT_FACTORED;
    for (auto &g : s->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    s->K = t.K;
    s->mrt = mrt;
    s->ops = ops;
    s->sp.assign(ops->step_size, 0);
    s->ep.assign(ops->eq_size, 0);
    ops->fill_step(s->sp.data(), h);
    ops->fill_eq(s->ep.data(), h);
    s->tau_bgk = h.omega > 0 ? 1.0 / h.omega : 1.0;
    if (collision == SCLBM_COLL_BGK && !coll_a && !(uniform_rate > 0)) s->tau_bgk = tau;
    if (s->noise_kind) {
        s->np.assign(ops->noise_size, 0);
        ops->fill_noise(s->np.data(), s->noise_kind, s->noise_indep, s->noise_m2var.data(), s->noise_coef.data());
        s->ngrid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)s->sms * ops->noise_occupancy(),
                                                               (s->V + 127) / 128));
    }
    ops->grids(s->sms, &s->dgrid, &s->fgrid);
    const int64_t need_d = (s->V + 255) / 256, need_f = (s->V + 127) / 128;
    s->dgrid = (int)std::max<int64_t>(1, std::min<int64_t>(s->dgrid, need_d));
    s->fgrid = (int)std::max<int64_t>(1, std::min<int64_t>(s->fgrid, need_f));
    plan_fused(s);
    return SCLBM_OK;
}

// The single-pass kernel does not write the density array; readers of it
// first reduce the current populations (the reference's n array holds the
// density at the start of the last step; here it is always the current one).
int ensure_density(sclbm_sim *s) {
    if (s->dn_fresh || !s->pop_set) return SCLBM_OK;
    cudaError_t e = density_pass(s);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "density: %s", cudaGetErrorString(e));
    s->dn_fresh = true;
    return SCLBM_OK;
}

}  // namespace

// ============================================================================
extern "C" {

const char *sclbm_version(void) { return "sclbm 0.1 (sm_103a)"; }

const char *sclbm_status_string(int st) {
    switch (st) {
    case SCLBM_OK: return "ok";
    case SCLBM_ERR_ARG: return "invalid argument";
    case SCLBM_ERR_UNSUPPORTED: return "unsupported configuration";
    case SCLBM_ERR_CUDA: return "CUDA error";
    case SCLBM_ERR_STATE: return "call out of order";
    case SCLBM_ERR_NOMEM: return "out of device memory";
    case SCLBM_ERR_NODEVICE: return "no usable device";
    default: return "unknown status";
    }
}

const char *sclbm_last_error(void) { return g_err.c_str(); }

int sclbm_monomial_count(int dim) {
    if (dim == 2) return Mono<2>::K;
    if (dim == 3) return Mono<3>::K;
    return 0;
}

int sclbm_create(const sclbm_params *p, sclbm_sim **out) {
    g_err.clear();
    if (!p || !out) return fail(SCLBM_ERR_ARG, "null argument");
    *out = nullptr;
    if (p->dim != 2 && p->dim != 3) return fail(SCLBM_ERR_UNSUPPORTED, "dimension %d (2 or 3 supported)", p->dim);
    if (!p->xi || !p->w || !p->e || !p->we) return fail(SCLBM_ERR_ARG, "null stencil table");
    const int *cx = compiled_xi(p->dim, p->q);
    if (!cx) return fail(SCLBM_ERR_UNSUPPORTED, "lattice D%dQ%d not built (D2Q9, D3Q19)", p->dim, p->q);
    for (int i = 0; i < p->q * p->dim; i++)
        if (p->xi[i] != cx[i]) return fail(SCLBM_ERR_UNSUPPORTED, "lattice velocities differ from D%dQ%d", p->dim, p->q);
    const int order = stencil_order(p->dim, p->e, p->qe);
    if (!order) return fail(SCLBM_ERR_UNSUPPORTED, "force stencil (%d vectors) is not E4/E6/E8", p->qe);
    for (int d = 0; d < p->dim; d++)
        if (p->sizes[d] < 2 || p->sizes[d] > (1 << 24))
            return fail(SCLBM_ERR_ARG, "size[%d] = %d out of range [2, 2^24]", d, p->sizes[d]);
    if (p->psi_kind < 0 || p->psi_kind > 2) return fail(SCLBM_ERR_ARG, "psi_kind %d", p->psi_kind);
    if (p->precision != SCLBM_FP64 && p->precision != SCLBM_FP32_SHIFTED)
        return fail(SCLBM_ERR_ARG, "precision %d", p->precision);
    if (!(p->c2 > 0)) return fail(SCLBM_ERR_ARG, "c2 must be > 0");

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SCLBM_ERR_NODEVICE, "no CUDA device visible");
    }
    if (p->device < 0 || p->device >= ndev) return fail(SCLBM_ERR_ARG, "device %d of %d", p->device, ndev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p->device) != cudaSuccess) return fail(SCLBM_ERR_CUDA, "device properties");
    if (prop.major < 10) return fail(SCLBM_ERR_NODEVICE, "device %s is sm_%d%d; built for sm_103a", prop.name,
                                     prop.major, prop.minor);

    if (p->collision != SCLBM_COLL_BGK && p->collision != SCLBM_COLL_MRT)
        return fail(SCLBM_ERR_ARG, "collision %d", p->collision);
    sclbm_sim *s = new sclbm_sim();
    s->device = p->device;
    DevGuard dg(s->device);
    s->D = p->dim;
    s->Q = p->q;
    s->QE = p->qe;
    s->order = order;
    s->V = 1;
    for (int d = 0; d < s->D; d++) {
        s->L[d] = p->sizes[d];
        s->V *= p->sizes[d];
    }
    s->fp32 = p->precision == SCLBM_FP32_SHIFTED;
    s->rs = s->fp32 ? 4 : 8;
    s->rho0 = s->fp32 ? p->rho0 : 0.0;
    s->c2 = p->c2;
    s->G = p->sc_g;
    s->psi_kind = p->psi_kind;
    s->literals = p->literals;
    s->sms = prop.multiProcessorCount;
    {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, p->device) != cudaSuccess) v = 0;
        cudaGetLastError();
        s->pageable_access = v == 1;
    }
    s->w.assign(p->w, p->w + p->q);
    s->we.assign(p->we, p->we + p->qe);
    s->sym_weights = weights_symmetric(p);
    s->xi.assign(p->xi, p->xi + p->q * p->dim);
    s->e.assign(p->e, p->e + p->qe * p->dim);
    {
        int rc0 = configure(s, p->collision, p->tau, p->mrt_s, p->coll_a, p->coll_b);
        if (rc0) {
            delete s;
            return rc0;
        }
    }

    int rc = SCLBM_OK;
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(SCLBM_ERR_CUDA, "stream create");
    }
    const size_t pb = (size_t)s->V * s->Q * s->rs, fb = (size_t)s->V * s->rs;
    if (!rc) rc = alloc(s, &s->pop[0], pb);
    if (!rc) rc = alloc(s, &s->pop[1], pb);
    if (!rc) rc = alloc(s, &s->dn, fb);
    if (!rc) rc = alloc(s, &s->psi, fb);
    if (!rc) rc = alloc(s, &s->u, fb * s->D);
    if (!rc) rc = alloc(s, &s->u_old, fb * s->D);
    s->red_blocks = prop.multiProcessorCount * 2;
    if (!rc) rc = alloc(s, (void **)&s->red, (size_t)s->red_blocks * 8 * sizeof(double));
    if (!rc) {
        // a host int the kernels can write (mapped pinned memory): the flag of
        // a bounded device wait that gave up, read after every synchronisation
        if (cudaHostAlloc((void **)&s->flag_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&s->flag_dev, s->flag_host, 0) != cudaSuccess) {
            cudaGetLastError();
            rc = fail(SCLBM_ERR_CUDA, "mapped flag");
        } else {
            *s->flag_host = 0;
            s->fg.err = s->flag_dev;
        }
    }
    if (!rc) {
        if (cudaMemsetAsync(s->u, 0, fb * s->D, s->st) != cudaSuccess ||
            cudaMemsetAsync(s->u_old, 0, fb * s->D, s->st) != cudaSuccess ||
            cudaMemsetAsync(s->dn, 0, fb, s->st) != cudaSuccess ||
            cudaStreamSynchronize(s->st) != cudaSuccess)
            rc = fail(SCLBM_ERR_CUDA, "memset: %s", cudaGetErrorString(cudaGetLastError()));
    }
    if (rc) {
        release(s);
        delete s;
        return rc;
    }
    *out = s;
    return SCLBM_OK;
}

int sclbm_destroy(sclbm_sim *s) {
    if (!s) return SCLBM_OK;
    {
        DevGuard dg(s->device);
        cudaStreamSynchronize(s->st);
        release(s);
    }
    delete s;
    return SCLBM_OK;
}

int sclbm_info(const sclbm_sim *s, int64_t *volume, int64_t *device_bytes) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (volume) *volume = s->V;
    if (device_bytes) *device_bytes = s->device_bytes;
    return SCLBM_OK;
}

int sclbm_kernels_per_step(const sclbm_sim *s, int *count) {
    if (!s || !count) return fail(SCLBM_ERR_ARG, "null argument");
    *count = s->simple_mode ? simple_kernels(s) : fused_path(s) ? 1 : 2;
    return SCLBM_OK;
}

int sclbm_set_collision(sclbm_sim *s, int collision, double tau, const double *mrt_s, const double *coll_a,
                        const double *coll_b) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return configure(s, collision, tau, mrt_s, coll_a, coll_b);
}

int sclbm_set_density(sclbm_sim *s, const double *n) {
    if (!s || !n) return fail(SCLBM_ERR_ARG, "null argument");
    DevGuard dg(s->device);
    double shift = s->rho0;
    int rc = h2d_real(s, s->dn, n, s->V, s->fp32 ? &shift : nullptr, s->V);
    if (!rc) s->n_set = s->dn_fresh = true;
    return rc;
}

int sclbm_set_velocity(sclbm_sim *s, const double *u) {
    if (!s || !u) return fail(SCLBM_ERR_ARG, "null argument");
    DevGuard dg(s->device);
    int rc = h2d_real(s, s->u, u, s->V * s->D, nullptr, s->V);
    if (!rc) s->u_set = true;
    return rc;
}

int sclbm_get_density(sclbm_sim *s, double *n) {
    if (!s || !n) return fail(SCLBM_ERR_ARG, "null argument");
    DevGuard dg(s->device);
    int rc = ensure_density(s);
    if (rc) return rc;
    double shift = s->rho0;
    return d2h_real(s, s->dn, n, s->V, s->fp32 ? &shift : nullptr, s->V);
}

int sclbm_get_velocity(sclbm_sim *s, double *u) {
    if (!s || !u) return fail(SCLBM_ERR_ARG, "null argument");
    DevGuard dg(s->device);
    return d2h_real(s, s->u, u, s->V * s->D, nullptr, s->V);
}

int sclbm_get_populations(sclbm_sim *s, double *pop) {
    if (!s || !pop) return fail(SCLBM_ERR_ARG, "null argument");
    DevGuard dg(s->device);
    std::vector<double> shift(s->Q);
    for (int q = 0; q < s->Q; q++) shift[q] = s->w[q] * s->rho0;
    return d2h_real(s, s->pop[s->cur], pop, s->V * s->Q, s->fp32 ? shift.data() : nullptr, s->V);
}

int sclbm_set_populations(sclbm_sim *s, const double *pop) {
    if (!s || !pop) return fail(SCLBM_ERR_ARG, "null argument");
    DevGuard dg(s->device);
    std::vector<double> shift(s->Q);
    for (int q = 0; q < s->Q; q++) shift[q] = s->w[q] * s->rho0;
    int rc = h2d_real(s, s->pop[s->cur], pop, s->V * s->Q, s->fp32 ? shift.data() : nullptr, s->V);
    if (!rc) {
        s->pop_set = true;
        s->moments_fresh = s->dn_fresh = false;
    }
    return rc;
}

int sclbm_init_populations(sclbm_sim *s) {
    // n and u start at zero after create, as the reference's zero-filled arrays
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    return init_pop(s);
}

int sclbm_init_radial(sclbm_sim *s, double n_g, double n_l, double R, int full_flag) {
    return profile(s, PROF_RADIAL, n_g, n_l, R, 0, 0, full_flag ? 1 : 0);
}
int sclbm_init_flat(sclbm_sim *s, double n_g, double n_l, double width, int direction, int full_flag) {
    return profile(s, PROF_FLAT, n_g, n_l, 0, width, direction, full_flag ? 1 : 0);
}
int sclbm_init_single_flat(sclbm_sim *s, double n_g, double n_l, int direction, int full_flag) {
    return profile(s, PROF_SINGLE_FLAT, n_g, n_l, 0, 0, direction, full_flag ? 1 : 0);
}
int sclbm_init_cylinder(sclbm_sim *s, double n_g, double n_l, double R, int direction, int full_flag) {
    return profile(s, PROF_CYLINDER, n_g, n_l, R, 0, direction, full_flag ? 1 : 0);
}

int sclbm_step(sclbm_sim *s, int64_t nsteps) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (nsteps < 0) return fail(SCLBM_ERR_ARG, "nsteps < 0");
    if (!s->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(s->device);
    // the simple family leaves in n and u what the reference's loops leave there
    // (the moments at the start of the last step, the stored velocity)
    const bool keep = s->simple_mode && nsteps > 0;
    if (!keep) s->moments_fresh = s->dn_fresh = false;
    const int rc = run_steps(s, nsteps);
    if (keep && !rc) s->moments_fresh = s->dn_fresh = true;
    return rc;
}

// after a synchronisation: a staged kernel's bounded wait that gave up
int check_flag(sclbm_sim *s) {
    if (s->flag_host && *(volatile int *)s->flag_host) {
        *s->flag_host = 0;
        return fail(SCLBM_ERR_CUDA, "a single-pass kernel gave up waiting on an mbarrier (TMA staging or the "
                                    "mbarrier psi ring); results of the last steps are invalid");
    }
    return SCLBM_OK;
}

int sclbm_selftest_bounded_wait(int device, int polls, int *gave_up, double *ms) {
    clear_error();
    if (!gave_up || polls < 1 || polls > MBAR_POLLS)
        return fail(SCLBM_ERR_ARG, "polls %d (1 .. %d), gave_up required", polls, MBAR_POLLS);
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return fail(SCLBM_ERR_NODEVICE, "device %d", device);
    }
    DevGuard dg(device);
    int *err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc((void **)&err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0);
    if (e == cudaSuccess) {
        k_bounded_wait_selftest<<<1, 32>>>(err, polls);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flag, err, sizeof(int), cudaMemcpyDeviceToHost);
    float t = 0.f;
    if (e == cudaSuccess && ms) e = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (err) cudaFree(err);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "bounded-wait self-test: %s", cudaGetErrorString(e));
    *gave_up = flag;
    if (ms) *ms = t;
    return SCLBM_OK;
}

int sclbm_sync(sclbm_sim *s) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return check_flag(s);
}

int sclbm_step_timed(sclbm_sim *s, int64_t nsteps, double *ms) {
    if (!s || !ms) return fail(SCLBM_ERR_ARG, "null argument");
    if (!s->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(s->device);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventRecord(e0, s->st));
    int rc = run_steps(s, nsteps);
    cudaEventRecord(e1, s->st);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->moments_fresh = s->dn_fresh = s->simple_mode && nsteps > 0 && rc == SCLBM_OK;
    *ms = t;
    if (rc) return rc;
    CUDA_TRY(cudaGetLastError());
    return check_flag(s);
}

int sclbm_profile_step(sclbm_sim *s, int64_t nsteps, double *ms, int nms) {
    if (!s || !ms || nms < 2) return fail(SCLBM_ERR_ARG, "bad argument");
    if (!s->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    if (nsteps < 1 || nsteps > 4096) return fail(SCLBM_ERR_ARG, "nsteps in [1, 4096]");
    if (s->simple_mode) return fail(SCLBM_ERR_UNSUPPORTED, "per-kernel times of the simple step family");
    DevGuard dg(s->device);
    // per step: an event before the step, then one after each kernel
    std::vector<cudaEvent_t> ev((size_t)nsteps * 3);
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    const bool fused = fused_path(s);
    int rc = SCLBM_OK;
    for (int64_t i = 0; i < nsteps && rc == SCLBM_OK; i++) {
        cudaEventRecord(ev[3 * i], s->st);
        rc = launch_step(s, &ev[3 * i + 1]);
    }
    cudaError_t ce = cudaStreamSynchronize(s->st);
    double t0 = 0, t1 = 0;
    for (int64_t i = 0; i < nsteps && ce == cudaSuccess && rc == SCLBM_OK; i++) {
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]);
        if (!fused) cudaEventElapsedTime(&b, ev[3 * i + 1], ev[3 * i + 2]);
        if (fused) t1 += a;
        else {
            t0 += a;
            t1 += b;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    s->moments_fresh = s->dn_fresh = false;
    if (rc) return rc;
    if (ce != cudaSuccess) return fail(SCLBM_ERR_CUDA, "profile: %s", cudaGetErrorString(ce));
    if ((rc = check_flag(s))) return rc;
    ms[0] = t0 / nsteps;  // density + psi pass (0 on the single-pass path)
    ms[1] = t1 / nsteps;  // force + collide + stream (the whole step on the single-pass path)
    return SCLBM_OK;
}

int sclbm_set_tuning(sclbm_sim *s, int path, int chunk) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (path < SCLBM_PATH_AUTO || path > SCLBM_PATH_FUSED_PAIRS) return fail(SCLBM_ERR_ARG, "path %d", path);
    const bool one_pass = path >= SCLBM_PATH_FUSED;
    if (one_pass && !s->ops->fused)
        return fail(SCLBM_ERR_UNSUPPORTED, "single-pass kernel is built for FP32-shifted storage only");
    if (one_pass && !s->sym_weights)
        return fail(SCLBM_ERR_UNSUPPORTED, "single-pass kernel needs equal weights on opposite directions");
    if (one_pass && !fused_fits(s))
        return fail(SCLBM_ERR_UNSUPPORTED, "single-pass kernel needs q*volume < 2^31");
    DevGuard dg(s->device);
    CUDA_TRY(cudaStreamSynchronize(s->st));
    s->path = path;
    s->chunk_override = chunk > 0 ? chunk : 0;
    plan_fused(s);
    for (auto &g : s->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    return SCLBM_OK;
}

int sclbm_get_tuning(const sclbm_sim *s, int *path, int *chunk, int *grid) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (path)
        *path = !fused_path(s)               ? SCLBM_PATH_TWO_PASS
                : s->fg.pairs && !s->walls ? SCLBM_PATH_FUSED_PAIRS
                                             : SCLBM_PATH_FUSED;
    if (chunk) *chunk = fused_path(s) ? s->fg.chunk : 0;
    if (grid) *grid = fused_path(s) ? s->fused_grid : s->fgrid;
    return SCLBM_OK;
}

int sclbm_set_tuning_ex(sclbm_sim *s, const sclbm_tuning *t) {
    if (!s || !t) return fail(SCLBM_ERR_ARG, "null argument");
    if (t->staging < -1 || t->staging > (SCLBM_STAGE_HALO_ASYNC | SCLBM_STAGE_OWN_TMA))
        return fail(SCLBM_ERR_ARG, "staging %d", t->staging);
    if (t->tile < -1 || t->tile >= N_TILES) return fail(SCLBM_ERR_ARG, "tile %d (0 .. %d)", t->tile, N_TILES - 1);
    if (t->order < -1 || t->order > 2) return fail(SCLBM_ERR_ARG, "order %d (0 .. 2)", t->order);
    const int saved = s->staging, saved_tile = s->tile, saved_order = s->item_order;
    s->staging = t->staging;
    s->tile = t->tile;
    s->item_order = t->order;
    const int rc = sclbm_set_tuning(s, t->path, t->chunk);
    if (rc) {
        s->staging = saved;
        s->tile = saved_tile;
        s->item_order = saved_order;
    }
    return rc;
}

int sclbm_get_tuning_ex(const sclbm_sim *s, sclbm_tuning *t) {
    if (!s || !t) return fail(SCLBM_ERR_ARG, "null argument");
    sclbm_get_tuning(s, &t->path, &t->chunk, &t->grid);
    t->staging = fused_path(s) ? s->fg.stg : 0;
    t->tile = fused_path(s) ? s->fg.tile : 0;
    t->order = fused_path(s) ? s->fg.order : 0;
    return SCLBM_OK;
}

// Autotuner (no counterpart in the reference, whose generated kernels run a
// fixed 128-thread block, idpy/LBM/MultiPhase.py:2072-2085).  Candidates are
// the variants of the handle's current step that compute bit-identical
// results: on the single pass, one or two halo cells per load, the staging
// flags and the chunk length (planes each CTA marches, i.e. cells per thread
// along the marching axis); the two-pass path has no variants.  Each is timed
// with CUDA events on the handle's stream over trial_steps launches that all
// read the current populations and write the other buffer (the state is left
// as it was); the fastest is applied and cached for this key.
int sclbm_autotune(sclbm_sim *s, int trial_steps, sclbm_tuning *best, double *best_ms) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (trial_steps < 1 || trial_steps > 10000) return fail(SCLBM_ERR_ARG, "trial_steps in [1, 10000]");
    if (!s->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    if (s->noise_kind)
        return fail(SCLBM_ERR_UNSUPPORTED, "fluctuating handles are not tuned (a trial step would advance the "
                                           "generator states)");
    if (s->simple_mode)
        return fail(SCLBM_ERR_UNSUPPORTED, "the simple step family is not tuned (its inlet/outlet kernels "
                                           "write the current populations)");
    DevGuard dg(s->device);
    CUDA_TRY(cudaStreamSynchronize(s->st));
    const int saved_path = s->path, saved_chunk = s->chunk_override, saved_stg = s->staging, saved_tile = s->tile,
              saved_order = s->item_order;
    struct Cand {
        int path, chunk, staging, tile, order;
    };
    std::vector<Cand> cands;
    if (!fused_path(s)) {
        cands.push_back({s->path, 0, 0, 0, 0});
    } else {
        const int Lm = s->D == 3 ? s->L[2] : s->L[1];
        const bool pairs_ok = s->D == 3 && s->L[0] % 2 == 0 && s->ops->fused_r % 2 == 0 && !s->walls;
        std::vector<int> chunks = {0};
        for (int c : {8, 12, 16, 24, 32, 40, 48, 64, 96, 128})
            if (c < Lm) chunks.push_back(c);
        std::vector<int> paths = {SCLBM_PATH_FUSED};
        if (pairs_ok) paths.insert(paths.begin(), SCLBM_PATH_FUSED_PAIRS);
        for (int path : paths) {
            for (int stg = 0; stg <= 3; stg++) {
                if (stg && (path != SCLBM_PATH_FUSED_PAIRS || !(s->ops->fused_stg_mask & stg))) continue;
                for (int c : chunks) cands.push_back({path, c, stg, 0, 0});
            }
            if (path == SCLBM_PATH_FUSED_PAIRS)
                for (int tile = 1; tile < N_TILES; tile++)
                    if (s->ops->fused_tile_mask >> tile & 1)
                        for (int c : chunks) cands.push_back({path, c, 0, tile, 0});
        }
    }
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    double best_t = 1e300;
    Cand win = cands[0];
    std::vector<std::array<int, 6>> seen;  // effective (pairs, staging, tile, chunk, grid, order) already timed
    int rc = SCLBM_OK;
    // two stages: every variant in the default item order, then the other
    // orders of the winner
    bool orders_added = false;
    for (size_t ci = 0; ci < cands.size(); ci++) {
        const Cand c = cands[ci];
        s->path = c.path;
        s->chunk_override = c.chunk;
        s->staging = c.staging;
        s->tile = c.tile;
        s->item_order = c.order;
        plan_fused(s);
        const bool fp = fused_path(s);
        const std::array<int, 6> eff = {fp ? s->fg.pairs : -1, fp ? s->fg.stg : -1, fp ? s->fg.tile : -1,
                                        fp ? s->fg.chunk : 0, fp ? s->fused_grid : 0, fp ? s->fg.order : 0};
        if (std::find(seen.begin(), seen.end(), eff) != seen.end()) continue;
        seen.push_back(eff);
        // one untimed launch, then trial_steps timed ones, all from the current buffer
        for (int i = 0; i <= trial_steps && rc == SCLBM_OK; i++) {
            if (i == 1) cudaEventRecord(e0, s->st);
            rc = launch_step(s);
            s->cur ^= 1;
        }
        cudaEventRecord(e1, s->st);
        const cudaError_t ce = cudaEventSynchronize(e1);
        if (rc == SCLBM_OK && ce != cudaSuccess) rc = fail(SCLBM_ERR_CUDA, "autotune: %s", cudaGetErrorString(ce));
        if (rc == SCLBM_OK) rc = check_flag(s);
        if (rc) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_t) {
            best_t = ms;
            win = c;
        }
        if (ci + 1 == cands.size() && !orders_added && fused_path(s) && cands.size() > 1) {
            orders_added = true;
            for (int order = 1; order <= 2; order++) cands.push_back({win.path, win.chunk, win.staging, win.tile, order});
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->moments_fresh = s->dn_fresh = false;
    if (rc) {
        s->path = saved_path;
        s->chunk_override = saved_chunk;
        s->staging = saved_stg;
        s->tile = saved_tile;
        s->item_order = saved_order;
        plan_fused(s);
        return rc;
    }
    s->path = win.path;
    s->chunk_override = win.chunk;
    s->staging = win.staging;
    s->tile = win.tile;
    s->item_order = win.order;
    plan_fused(s);
    for (auto &g : s->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    sclbm_tuning t = {};
    sclbm_get_tuning_ex(s, &t);
    t.chunk = win.chunk;  // 0: the planner's choice won (re-planned for the box)
    t.path = win.path;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[tune_key(s)] = t;
    }
    if (best) sclbm_get_tuning_ex(s, best);
    if (best_ms) *best_ms = best_t / trial_steps;
    return SCLBM_OK;
}

int sclbm_clear_tuning_cache(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
    return SCLBM_OK;
}

int sclbm_compute_moments(sclbm_sim *s) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (!s->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(s->device);
    cudaError_t e = density_pass(s);
    if (e == cudaSuccess) e = s->ops->velocity(s->pop[s->cur], s->dn, s->psi, s->u, s->sp.data(), s->fgrid, s->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "moments: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    s->n_set = s->u_set = true;
    s->moments_fresh = s->dn_fresh = true;
    return SCLBM_OK;
}

int sclbm_reductions(sclbm_sim *s, double *mass, double *momentum) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (!s->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(s->device);
    const int nv = 1 + s->D;
    if (s->D == 2) {
        if (s->fp32) k_reduce_pop<D2Q9, float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const float *)s->pop[s->cur], s->V, s->rho0, s->red);
        else k_reduce_pop<D2Q9, double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const double *)s->pop[s->cur], s->V, 0.0, s->red);
    } else {
        if (s->fp32) k_reduce_pop<D3Q19, float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const float *)s->pop[s->cur], s->V, s->rho0, s->red);
        else k_reduce_pop<D3Q19, double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const double *)s->pop[s->cur], s->V, 0.0, s->red);
    }
    std::vector<double> part;
    int rc = finish_partials(s, nv, part);
    if (rc) return rc;
    double acc[4] = {0, 0, 0, 0};
    for (int b = 0; b < s->red_blocks; b++)
        for (int i = 0; i < nv; i++) acc[i] += part[(size_t)b * nv + i];
    if (mass) *mass = acc[0];
    if (momentum)
        for (int d = 0; d < s->D; d++) momentum[d] = acc[1 + d];
    return SCLBM_OK;
}

int sclbm_check_u(sclbm_sim *s, double *u_conv, double *max_u) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (!s->moments_fresh) return fail(SCLBM_ERR_STATE, "call sclbm_compute_moments first");
    DevGuard dg(s->device);
    if (s->fp32) k_check_u<float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const float *)s->u, (float *)s->u_old, s->D, s->V, s->red);
    else k_check_u<double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const double *)s->u, (double *)s->u_old, s->D, s->V, s->red);
    std::vector<double> part;
    int rc = finish_partials(s, 2, part);
    if (rc) return rc;
    double sum = 0, mx = 0;
    for (int b = 0; b < s->red_blocks; b++) {
        sum += part[(size_t)b * 2];
        mx = std::max(mx, part[(size_t)b * 2 + 1]);
    }
    if (u_conv) *u_conv = sum / (double)s->V;
    if (max_u) *max_u = std::sqrt(mx / s->c2);
    return SCLBM_OK;
}

int sclbm_center_of_mass(sclbm_sim *s, double *mass, double *cm) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    {
        int rc0 = ensure_density(s);
        if (rc0) return rc0;
    }
    if (s->fp32) k_com<float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const float *)s->dn, s->rho0, s->D, s->L[0], s->L[1], s->V, s->red);
    else k_com<double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const double *)s->dn, 0.0, s->D, s->L[0], s->L[1], s->V, s->red);
    std::vector<double> part;
    int rc = finish_partials(s, 4, part);
    if (rc) return rc;
    double acc[4] = {0, 0, 0, 0};
    for (int b = 0; b < s->red_blocks; b++)
        for (int i = 0; i < 4; i++) acc[i] += part[(size_t)b * 4 + i];
    if (mass) *mass = acc[0];
    if (cm)
        for (int d = 0; d < s->D; d++) cm[d] = acc[1 + d] / acc[0];
    return SCLBM_OK;
}

int sclbm_density_at(sclbm_sim *s, const int64_t *idx, int count, double *out) {
    if (!s || !idx || !out || count < 0) return fail(SCLBM_ERR_ARG, "bad argument");
    DevGuard dg(s->device);
    {
        int rc0 = ensure_density(s);
        if (rc0) return rc0;
    }
    for (int i = 0; i < count; i++) {
        if (idx[i] < 0 || idx[i] >= s->V) return fail(SCLBM_ERR_ARG, "index %lld out of range", (long long)idx[i]);
        if (s->fp32) {
            float v;
            CUDA_TRY(cudaMemcpyAsync(&v, (const float *)s->dn + idx[i], 4, cudaMemcpyDeviceToHost, s->st));
            CUDA_TRY(cudaStreamSynchronize(s->st));
            out[i] = (double)v + s->rho0;
        } else {
            CUDA_TRY(cudaMemcpyAsync(out + i, (const double *)s->dn + idx[i], 8, cudaMemcpyDeviceToHost, s->st));
            CUDA_TRY(cudaStreamSynchronize(s->st));
        }
    }
    return SCLBM_OK;
}

int sclbm_set_walls(sclbm_sim *s, const int *walls, const double *psi) {
    if (!s || !walls || !psi) return fail(SCLBM_ERR_ARG, "null argument");
    if (s->noise_kind) return fail(SCLBM_ERR_UNSUPPORTED, "walls with fluctuations (the reference has no such step)");
    for (int64_t g = 0; g < s->V; g++)
        if (walls[g] < 0 || walls[g] > 3)
            return fail(SCLBM_ERR_ARG, "walls[%lld] = %d (1 fluid, 0 wall, 2 inlet, 3 outlet)", (long long)g,
                        walls[g]);
    DevGuard dg(s->device);
    int rc = SCLBM_OK;
    if (!s->walls) rc = alloc(s, (void **)&s->walls, (size_t)s->V);
    if (!rc && !s->psi_w) rc = alloc(s, &s->psi_w, (size_t)s->V * s->rs);
    if (rc) return rc;
    std::vector<unsigned char> w(s->V);
    for (int64_t g = 0; g < s->V; g++) w[g] = (unsigned char)walls[g];
    CUDA_TRY(cudaMemcpyAsync(s->walls, w.data(), s->V, cudaMemcpyHostToDevice, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    // the walls' psi, and the psi array as the reference's GetWalls leaves it
    rc = h2d_real(s, s->psi_w, psi, s->V, nullptr, 0);
    if (!rc) rc = h2d_real(s, s->psi, psi, s->V, nullptr, 0);
    if (rc) return rc;
    for (auto &g : s->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;  // the step's kernels change
    s->moments_fresh = s->dn_fresh = false;
    plan_fused(s);  // the single pass with walls has its own occupancy
    return SCLBM_OK;
}

int sclbm_noise_counts(int dim, int q, int indep, int *moments, int *streams) {
    if (dim < 1 || q <= dim + 1) return fail(SCLBM_ERR_ARG, "dim %d, q %d", dim, q);
    const int nr = q - dim - 1;
    if (moments) *moments = nr;
    if (streams) *streams = indep ? 2 * nr : nr;
    return SCLBM_OK;
}

int sclbm_noise_operator(const sclbm_params *p, double kBT, double n0, double *m2var, double *coef) {
    if (!p || !p->xi || !p->w || !m2var || !coef) return fail(SCLBM_ERR_ARG, "null argument");
    if ((p->dim != 2 && p->dim != 3) || p->q <= p->dim + 1) return fail(SCLBM_ERR_ARG, "dim %d, q %d", p->dim, p->q);
    if (!(p->tau > 0) || !(kBT >= 0) || !std::isfinite(kBT) || !std::isfinite(n0))
        return fail(SCLBM_ERR_ARG, "tau %g, kBT %g, n0 %g", p->tau, kBT, n0);
    CollisionSpec cs;
    cs.dim = p->dim;
    cs.q = p->q;
    cs.xi = p->xi;
    cs.w = p->w;
    cs.c2 = p->c2;
    cs.tau = p->tau;
    cs.literals = p->literals;
    std::vector<double> mv, cf;
    std::string err;
    if (build_noise(cs, kBT, n0, mv, cf, err)) return fail(SCLBM_ERR_UNSUPPORTED, "noise operator: %s", err.c_str());
    std::copy(mv.begin(), mv.end(), m2var);
    std::copy(cf.begin(), cf.end(), coef);
    return SCLBM_OK;
}

int sclbm_set_fluctuations(sclbm_sim *s, int generator, int indep, double kBT, double n0, const void *seeds,
                           int layout, const double *m2var, const double *coef) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    CUDA_TRY(cudaStreamSynchronize(s->st));
    for (auto &g : s->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;  // the step's kernels change
    if (generator == SCLBM_CRNG_NONE) {
        if (s->seeds) cudaFree(s->seeds), s->device_bytes -= (int64_t)s->noise_streams * s->V *
                                                             (s->noise_kind == SCLBM_CRNG_MMIX ? 8 : 4);
        s->seeds = nullptr;
        s->noise_kind = s->noise_streams = 0;
        plan_fused(s);
        return SCLBM_OK;
    }
    if (generator != SCLBM_CRNG_MINSTD && generator != SCLBM_CRNG_NUMREC && generator != SCLBM_CRNG_MMIX)
        return fail(SCLBM_ERR_ARG, "generator %d", generator);
    if (!seeds) return fail(SCLBM_ERR_ARG, "null seeds");
    if (layout != SCLBM_SEEDS_STREAM_MAJOR && layout != SCLBM_SEEDS_CELL_MAJOR)
        return fail(SCLBM_ERR_ARG, "seeds layout %d", layout);
    if ((m2var == nullptr) != (coef == nullptr)) return fail(SCLBM_ERR_ARG, "m2var and coef go together");
    if (s->mrt || !s->ops->fcs_noise) return fail(SCLBM_ERR_UNSUPPORTED, "the fluctuating step is BGK only");
    if (s->walls) return fail(SCLBM_ERR_UNSUPPORTED, "walls with fluctuations (the reference has no such step)");
    if (s->simple_mode) return fail(SCLBM_ERR_UNSUPPORTED, "fluctuations with the simple step family");
    if (!(kBT >= 0) || !std::isfinite(kBT) || !std::isfinite(n0)) return fail(SCLBM_ERR_ARG, "kBT %g, n0 %g", kBT, n0);
    const int nr = s->Q - s->D - 1, ns = indep ? 2 * nr : nr;
    std::vector<double> mv, cf;
    if (m2var) {
        mv.assign(m2var, m2var + nr);
        cf.assign(coef, coef + (size_t)s->Q * nr);
    } else {
        CollisionSpec cs;
        cs.dim = s->D;
        cs.q = s->Q;
        cs.xi = s->xi.data();
        cs.w = s->w.data();
        cs.c2 = s->c2;
        cs.tau = s->tau_bgk;
        cs.literals = s->fp32 ? SCLBM_LIT_EXACT : s->literals;
        std::string err;
        if (build_noise(cs, kBT, n0, mv, cf, err)) return fail(SCLBM_ERR_UNSUPPORTED, "noise operator: %s", err.c_str());
    }
    for (double v : mv)
        if (!std::isfinite(v) || v > 0) return fail(SCLBM_ERR_ARG, "m2var must be finite and <= 0");
    // generator states: uint64 for MMIX, uint32 otherwise; stored stream-major
    const size_t es = generator == SCLBM_CRNG_MMIX ? 8 : 4;
    const size_t bytes = (size_t)ns * s->V * es;
    if (s->seeds && (size_t)s->noise_streams * s->V * (s->noise_kind == SCLBM_CRNG_MMIX ? 8 : 4) != bytes) {
        cudaFree(s->seeds);
        s->device_bytes -= (int64_t)s->noise_streams * s->V * (s->noise_kind == SCLBM_CRNG_MMIX ? 8 : 4);
        s->seeds = nullptr;
    }
    if (!s->seeds) {
        int rc = alloc(s, &s->seeds, bytes);
        if (rc) return rc;
    }
    std::vector<unsigned char> host(bytes);
    for (int64_t g = 0; g < s->V; g++)
        for (int k = 0; k < ns; k++) {
            const size_t src = layout == SCLBM_SEEDS_STREAM_MAJOR ? (size_t)k * s->V + g : (size_t)g * ns + k;
            const size_t dst = (size_t)k * s->V + g;
            std::memcpy(host.data() + dst * es, (const unsigned char *)seeds + src * es, es);
        }
    CUDA_TRY(cudaMemcpyAsync(s->seeds, host.data(), bytes, cudaMemcpyHostToDevice, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    s->noise_kind = generator;
    s->noise_indep = indep ? 1 : 0;
    s->noise_streams = ns;
    s->noise_m2var = mv;
    s->noise_coef = cf;
    s->noise_sparse = true;
    for (int q = 0; q < s->Q; q++)
        for (int k = 0; k < nr; k++)
            if (cf[(size_t)q * nr + k] != 0.0 && !((s->ops->noise_mask(q) >> k) & 1u)) s->noise_sparse = false;
    s->np.assign(s->ops->noise_size, 0);
    s->ops->fill_noise(s->np.data(), s->noise_kind, s->noise_indep, mv.data(), cf.data());
    s->ngrid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)s->sms * s->ops->noise_occupancy(),
                                                           (s->V + 127) / 128));
    plan_fused(s);  // the fluctuating single-pass kernel has its own occupancy
    return SCLBM_OK;
}

int sclbm_get_seeds(sclbm_sim *s, void *seeds, int layout) {
    if (!s || !seeds) return fail(SCLBM_ERR_ARG, "null argument");
    if (!s->noise_kind) return fail(SCLBM_ERR_STATE, "no fluctuations set");
    if (layout != SCLBM_SEEDS_STREAM_MAJOR && layout != SCLBM_SEEDS_CELL_MAJOR)
        return fail(SCLBM_ERR_ARG, "seeds layout %d", layout);
    DevGuard dg(s->device);
    const size_t es = s->noise_kind == SCLBM_CRNG_MMIX ? 8 : 4, ns = (size_t)s->noise_streams;
    std::vector<unsigned char> host(ns * s->V * es);
    CUDA_TRY(cudaMemcpyAsync(host.data(), s->seeds, host.size(), cudaMemcpyDeviceToHost, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    for (int64_t g = 0; g < s->V; g++)
        for (size_t k = 0; k < ns; k++) {
            const size_t src = k * s->V + g;
            const size_t dst = layout == SCLBM_SEEDS_STREAM_MAJOR ? k * s->V + g : g * ns + k;
            std::memcpy((unsigned char *)seeds + dst * es, host.data() + src * es, es);
        }
    return SCLBM_OK;
}

int sclbm_set_simple(sclbm_sim *s, int forcing, int use_walls, int gravity, double g, int inlet_outlet,
                     double u_in) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    CUDA_TRY(cudaStreamSynchronize(s->st));
    for (auto &gr : s->graph)
        if (gr) cudaGraphExecDestroy(gr), gr = nullptr;  // the step's kernels change
    if (forcing == SCLBM_SIMPLE_OFF) {
        s->simple_mode = s->simple_inout = 0;
        return SCLBM_OK;
    }
    if (forcing != SCLBM_SIMPLE_GUO && forcing != SCLBM_SIMPLE_SC) return fail(SCLBM_ERR_ARG, "forcing %d", forcing);
    if (!s->ops->simple_collide) return fail(SCLBM_ERR_UNSUPPORTED, "no simple-step kernels");
    if (s->mrt) return fail(SCLBM_ERR_UNSUPPORTED, "the simple step family is BGK");
    if (s->noise_kind) return fail(SCLBM_ERR_UNSUPPORTED, "the simple step family with fluctuations");
    if (gravity && forcing != SCLBM_SIMPLE_GUO)
        return fail(SCLBM_ERR_UNSUPPORTED, "gravity goes with Guo forcing (MainLoopSimpleWallsGravity)");
    if (gravity && inlet_outlet) return fail(SCLBM_ERR_UNSUPPORTED, "gravity with inlet/outlet");
    if ((inlet_outlet || use_walls) && !s->walls) return fail(SCLBM_ERR_STATE, "no walls set (sclbm_set_walls)");
    if (inlet_outlet && !use_walls) return fail(SCLBM_ERR_ARG, "inlet/outlet flags are wall flags");
    if (!std::isfinite(g) || !std::isfinite(u_in)) return fail(SCLBM_ERR_ARG, "g %g, u_in %g", g, u_in);
    if (inlet_outlet) {
        // every outlet cell copies the cell at x - 1
        std::vector<unsigned char> w(s->V);
        CUDA_TRY(cudaMemcpyAsync(w.data(), s->walls, s->V, cudaMemcpyDeviceToHost, s->st));
        CUDA_TRY(cudaStreamSynchronize(s->st));
        for (int64_t c = 0; c < s->V; c++)
            if (w[c] == 3 && c % s->L[0] == 0) return fail(SCLBM_ERR_ARG, "outlet cell %lld at x = 0", (long long)c);
    }
    SimpleParams &p = s->spar;
    p = SimpleParams{};
    for (int d = 0; d < 3; d++) p.geo.L[d] = d < s->D ? s->L[d] : 1;
    p.geo.V = s->V;
    for (int q = 0; q < s->Q; q++) p.w[q] = s->w[q];
    for (int a = 0; a < s->QE; a++) p.we[a] = s->we[a];
    p.neg_g = -s->G;
    p.omega = 1.0 / s->tau_bgk;
    p.g = g;
    p.u_in = u_in;
    p.psi_kind = s->psi_kind;
    p.rho0 = s->fp32 ? s->rho0 : 0.0;
    p.gravity = gravity ? 1 : 0;
    s->simple_mode = forcing;
    s->simple_inout = inlet_outlet ? 1 : 0;
    s->simple_walls = use_walls ? 1 : 0;
    return SCLBM_OK;
}

int sclbm_set_transfer(sclbm_sim *s, int mode, int *pageable_access) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    if (mode != SCLBM_TRANSFER_AUTO && mode != SCLBM_TRANSFER_STAGED && mode != SCLBM_TRANSFER_DIRECT)
        return fail(SCLBM_ERR_ARG, "transfer mode %d", mode);
    s->transfer = mode;
    if (pageable_access) *pageable_access = s->pageable_access ? 1 : 0;
    return SCLBM_OK;
}

int sclbm_restore_mass(sclbm_sim *s, double target, double *before) {
    double m = 0;
    int rc = sclbm_reductions(s, &m, nullptr);
    if (rc) return rc;
    if (before) *before = m;
    if (!std::isfinite(target) || !std::isfinite(m)) return SCLBM_OK;
    DevGuard dg(s->device);
    const double delta = (target - m) / (double)s->V;
    if (s->fp32) {
        if ((float)delta == 0.f) return SCLBM_OK;
        k_add_rest<float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((float *)s->pop[s->cur], s->V, (float)delta);
    } else {
        if (delta == 0.0) return SCLBM_OK;
        k_add_rest<double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((double *)s->pop[s->cur], s->V, delta);
    }
    CUDA_TRY(cudaGetLastError());
    s->moments_fresh = s->dn_fresh = false;
    return SCLBM_OK;
}

int sclbm_density_finite(sclbm_sim *s, int *finite, double *max_abs) {
    if (!s) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(s->device);
    {
        int rc0 = ensure_density(s);
        if (rc0) return rc0;
    }
    if (s->fp32) k_finite<float><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const float *)s->dn, s->rho0, s->V, s->red);
    else k_finite<double><<<s->red_blocks, RED_THREADS, 0, s->st>>>((const double *)s->dn, 0.0, s->V, s->red);
    std::vector<double> part;
    int rc = finish_partials(s, 2, part);
    if (rc) return rc;
    double bad = 0, mx = 0;
    for (int b = 0; b < s->red_blocks; b++) {
        bad = std::max(bad, part[(size_t)b * 2]);
        mx = std::max(mx, part[(size_t)b * 2 + 1]);
    }
    if (finite) *finite = bad > 0 ? 0 : 1;
    if (max_abs) *max_abs = mx;
    return SCLBM_OK;
}

}  // extern "C"

// ============================================================================
// Batches of independent lattices (include/sclbm.h, sclbm_batch_*)
// ============================================================================
struct sclbm_batch {
    int device = 0, sms = 1;
    cudaStream_t st = nullptr;
    int D = 0, Q = 0, order = 0, n = 0;
    double c2 = 1.0 / 3;
    int psi_kind = 0;
    std::vector<int> sizes;
    std::vector<double> w;
    std::vector<BatchInst> inst;
    BatchInst *inst_d = nullptr;
    int64_t Vtot = 0;
    std::vector<int4> items;
    int4 *items_d = nullptr;
    size_t items_cap = 0;  // work items items_d holds
    int *counter = nullptr;  // [2] work queues, one per step parity
    float *wq_d = nullptr;
    const KernelOps *ops = nullptr;
    std::vector<unsigned char> sp;
    void *pop[2] = {nullptr, nullptr};
    int cur = 0;
    void *dn = nullptr, *psi = nullptr, *u_old = nullptr;
    double *partials = nullptr;
    double *probe_d = nullptr;  // [2n] centre / last-cell densities
    int probe_rad = 0;          // probes average the cube of side 2 rad + 1 about each cell
    float *delta_d = nullptr;   // [n] rest-population corrections
    int gx = 1, grid = 1, chunk = 32;
    int pairs = 0;          // 3D, even radius, every Lx and first cell even: paired halo loads
    int tx = 0;             // 2D tile width (0: the single-lattice kernel's; BATCH_TX_NARROW)
    int exact_rest = 1;     // compensated rest population (0: 3D paired BGK batches only)
    std::vector<int> home;  // buffer holding a retired lattice's state (-1 while active)
    std::vector<int64_t> steps;
    bool pop_set = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int64_t device_bytes = 0;
};

namespace {

constexpr int BATCH_CHUNK = 32;     // longest run of planes per work item
// shortest (items are re-planned as lattices retire): 2 rather than 4 took
// the step of a lone 224^2 D2Q9 E8 droplet from 8.3 to 6.3 us
constexpr int BATCH_MIN_CHUNK = 2;
constexpr int BATCH_CHECK_BLOCKS = 32;  // blocks per lattice in the observable kernels

int balloc(sclbm_batch *b, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(SCLBM_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    }
    b->device_bytes += (int64_t)bytes;
    return SCLBM_OK;
}

void brelease(sclbm_batch *b) {
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    for (void *p : {b->pop[0], b->pop[1], b->dn, b->psi, b->u_old, (void *)b->partials, (void *)b->inst_d,
                    (void *)b->items_d, (void *)b->counter, (void *)b->wq_d, (void *)b->probe_d,
                    (void *)b->delta_d})
        if (p) cudaFree(p);
    if (b->st) cudaStreamDestroy(b->st);
}

int64_t lattice_cells(const sclbm_batch *b, int i) {
    int64_t v = 1;
    for (int d = 0; d < b->D; d++) v *= b->sizes[(size_t)i * b->D + d];
    return v;
}

// Work items of the active lattices: tiles x runs of `chunk` marching planes.
// A work item's planes are processed one after another (each a global-memory
// round trip and a barrier), so the step time has a floor of about
// (chunk + 2R) plane latencies, while each item also re-reads 2R halo planes;
// batch_plan weighs the two.
void batch_items(const sclbm_batch *b, int chunk, std::vector<int4> &items) {
    items.clear();
    const int TX = b->tx ? b->tx : b->ops->fused_tx, TY = b->ops->fused_ty;
    for (int i = 0; i < b->n; i++) {
        if (!b->inst[i].active) continue;
        const BatchInst &I = b->inst[i];
        const int Lm = b->D == 3 ? I.Lz : I.Ly;
        for (int m0 = 0; m0 < Lm; m0 += chunk)
            for (int y0 = 0; y0 < (b->D == 3 ? I.Ly : 1); y0 += TY)
                for (int x0 = 0; x0 < I.Lx; x0 += TX)
                    items.push_back(make_int4(i, x0, y0, m0 | (std::min(m0 + chunk, Lm) << 16)));
    }
}

// The plane run per item: the one (of 32, 16, .., BATCH_MIN_CHUNK) with the
// fewest sequential plane passes per step, waves x (chunk + 2R), waves =
// items / resident CTAs rounded up; on a tie the longer run (less halo
// re-read).  Many cells: many waves, and the long run wins by its smaller
// halo share; few cells: one wave, and the run shrinks until a second wave
// would be needed.
int batch_plan(sclbm_batch *b) {
    const int resident = b->sms * b->ops->batch_occupancy(b->pairs, b->tx);
    const int R = b->ops->fused_r;
    int chunk = BATCH_CHUNK;
    int64_t best = -1;
    std::vector<int4> items, trial;
    for (int c = BATCH_CHUNK; c >= BATCH_MIN_CHUNK; c /= 2) {
        batch_items(b, c, trial);
        const int64_t waves = std::max<int64_t>(1, ((int64_t)trial.size() + resident - 1) / resident);
        const int64_t passes = waves * (c + 2 * R);
        if (best < 0 || passes < best) {
            best = passes;
            chunk = c;
            items.swap(trial);
        }
    }
    if (items.size() > b->items_cap)
        return fail(SCLBM_ERR_STATE, "%zu work items, room for %zu", items.size(), b->items_cap);
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;  // they hold the item count and grid
    b->items.swap(items);
    b->chunk = chunk;
    if (!b->items.empty())
        CUDA_TRY(cudaMemcpyAsync(b->items_d, b->items.data(), sizeof(int4) * b->items.size(), cudaMemcpyHostToDevice,
                                 b->st));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    b->grid = std::max(1, std::min((int)b->items.size(), resident));
    return SCLBM_OK;
}

int batch_launch_step(sclbm_batch *b) {
    cudaError_t e = b->ops->batch_step(b->pop[b->cur], b->pop[b->cur ^ 1], b->sp.data(), b->inst_d, b->items_d,
                                       (int)b->items.size(), (int)b->Vtot, b->counter, b->cur, b->pairs, b->tx, b->exact_rest, b->grid,
                                       b->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "batch step: %s", cudaGetErrorString(e));
    b->cur ^= 1;
    return SCLBM_OK;
}

int batch_run(sclbm_batch *b, int64_t nsteps) {
    // the queue of step s is counter[s parity]; a graph holds an even number of steps
    while (nsteps >= GRAPH_STEPS) {
        if (!b->graph[b->cur]) {
            const int saved = b->cur;
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
            int rc = SCLBM_OK;
            for (int i = 0; i < GRAPH_STEPS && rc == SCLBM_OK; i++) rc = batch_launch_step(b);
            cudaError_t ce = cudaStreamEndCapture(b->st, &g);
            b->cur = saved;
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (ce != cudaSuccess) return fail(SCLBM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
            ce = cudaGraphInstantiate(&b->graph[saved], g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return fail(SCLBM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
        }
        CUDA_TRY(cudaGraphLaunch(b->graph[b->cur], b->st));
        nsteps -= GRAPH_STEPS;
    }
    for (int64_t i = 0; i < nsteps; i++) {
        int rc = batch_launch_step(b);
        if (rc) return rc;
    }
    return SCLBM_OK;
}

}  // namespace

extern "C" {

int sclbm_batch_create(const sclbm_params *p, int n, const int *sizes, const double *G, const double *rho0,
                       sclbm_batch **out) {
    g_err.clear();
    if (!p || !out || !sizes || !G || !rho0 || n < 1) return fail(SCLBM_ERR_ARG, "bad argument");
    *out = nullptr;
    if (p->precision != SCLBM_FP32_SHIFTED) return fail(SCLBM_ERR_UNSUPPORTED, "batches use FP32-shifted storage");
    if (p->dim != 2 && p->dim != 3) return fail(SCLBM_ERR_UNSUPPORTED, "dimension %d", p->dim);
    if (!p->xi || !p->w || !p->e || !p->we) return fail(SCLBM_ERR_ARG, "null stencil table");
    const int *cx = compiled_xi(p->dim, p->q);
    if (!cx) return fail(SCLBM_ERR_UNSUPPORTED, "lattice D%dQ%d not built", p->dim, p->q);
    for (int i = 0; i < p->q * p->dim; i++)
        if (p->xi[i] != cx[i]) return fail(SCLBM_ERR_UNSUPPORTED, "lattice velocities differ");
    const int order = stencil_order(p->dim, p->e, p->qe);
    if (!order) return fail(SCLBM_ERR_UNSUPPORTED, "force stencil is not E4/E6/E8");
    if (!weights_symmetric(p))
        return fail(SCLBM_ERR_UNSUPPORTED, "batches need equal weights on opposite directions");
    if (p->collision != SCLBM_COLL_BGK || !(p->tau > 0))
        return fail(SCLBM_ERR_UNSUPPORTED, "batches run BGK with tau > 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SCLBM_ERR_NODEVICE, "no CUDA device visible");
    }
    if (p->device < 0 || p->device >= ndev) return fail(SCLBM_ERR_ARG, "device %d", p->device);
    int64_t Vtot = 0;
    for (int i = 0; i < n; i++) {
        int64_t v = 1;
        for (int d = 0; d < p->dim; d++) {
            const int L = sizes[(size_t)i * p->dim + d];
            if (L < 2 || L > 32767) return fail(SCLBM_ERR_ARG, "lattice %d size %d out of range", i, L);
            v *= L;
        }
        Vtot += v;
    }
    if ((int64_t)p->q * Vtot >= ((int64_t)1 << 31))
        return fail(SCLBM_ERR_UNSUPPORTED, "batch too large: q * cells must stay below 2^31");

    sclbm_batch *b = new sclbm_batch();
    b->device = p->device;
    DevGuard dg(b->device);
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, b->device);
    b->sms = prop.multiProcessorCount;
    b->D = p->dim;
    b->Q = p->q;
    b->order = order;
    b->n = n;
    b->c2 = p->c2;
    b->psi_kind = p->psi_kind;
    b->sizes.assign(sizes, sizes + (size_t)n * p->dim);
    b->w.assign(p->w, p->w + p->q);
    b->Vtot = Vtot;
    b->ops = select_ops(p->dim, order, false, true, false);
    b->home.assign(n, -1);
    b->steps.assign(n, 0);
    // lattices and work items (lattice-major so concurrent items are neighbours)
    int64_t base = 0;
    for (int i = 0; i < n; i++) {
        const int *L = &b->sizes[(size_t)i * b->D];
        BatchInst I;
        I.base = (int)base;
        I.Lx = L[0];
        I.Ly = L[1];
        I.Lz = b->D == 3 ? L[2] : 1;
        I.neg_g = (float)(-G[i]);
        I.rho0 = (float)rho0[i];
        I.active = 1;
        I.pad = 0;
        b->inst.push_back(I);
        base += lattice_cells(b, i);
    }
    // paired halo loads when every lattice keeps them aligned
    b->pairs = b->D == 3 && b->ops && b->ops->fused_r % 2 == 0 && Vtot % 2 == 0;
    for (const BatchInst &I : b->inst) b->pairs = b->pairs && I.Lx % 2 == 0 && I.base % 2 == 0;
    // step parameters (BGK, FP32); G and rho0 come from the lattice table
    CollisionSpec cs;
    cs.dim = b->D;
    cs.q = b->Q;
    cs.xi = p->xi;
    cs.w = p->w;
    cs.c2 = p->c2;
    cs.tau = p->tau;
    cs.literals = SCLBM_LIT_EXACT;
    CollisionTables t;
    std::string err;
    int rc = build_collision(cs, t, err) ? fail(SCLBM_ERR_UNSUPPORTED, "collision operator: %s", err.c_str())
                                         : SCLBM_OK;
    if (!rc) {
        HostSetup h = {};
        h.L[0] = h.L[1] = h.L[2] = 1;
        h.V = Vtot;
        h.psi_kind = p->psi_kind;
        h.we = p->we;
        h.A = t.A.data();
        h.B = t.B.data();
        h.Beq = t.Beq.data();
        h.a_nonzero = t.A[0] != 0.0;
        h.omega = 1.0 / p->tau;
        h.w = p->w;
        b->sp.assign(b->ops->step_size, 0);
        b->ops->fill_step(b->sp.data(), h);
    }
    const size_t pb = (size_t)Vtot * b->Q * 4, fb = (size_t)Vtot * 4;
    if (!rc && cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess)
        rc = fail(SCLBM_ERR_CUDA, "stream create");
    if (!rc) rc = balloc(b, &b->pop[0], pb);
    if (!rc) rc = balloc(b, &b->pop[1], pb);
    if (!rc) rc = balloc(b, &b->dn, fb);
    if (!rc) rc = balloc(b, &b->psi, fb);
    if (!rc) rc = balloc(b, &b->u_old, fb * b->D);
    b->gx = BATCH_CHECK_BLOCKS;
    if (!rc) rc = balloc(b, (void **)&b->partials, (size_t)n * b->gx * BATCH_NV * sizeof(double));
    if (!rc) rc = balloc(b, (void **)&b->inst_d, sizeof(BatchInst) * n);
    {
        // the longest item list: every lattice, the shortest chunk, the narrowest tiles
        std::vector<int4> most;
        b->tx = b->D == 2 ? BATCH_TX_NARROW : 0;
        batch_items(b, BATCH_MIN_CHUNK, most);
        b->tx = 0;
        b->items_cap = most.size();
        if (!rc) rc = balloc(b, (void **)&b->items_d, sizeof(int4) * most.size());
    }
    if (!rc) rc = balloc(b, (void **)&b->counter, 2 * sizeof(int));
    if (!rc) rc = balloc(b, (void **)&b->wq_d, sizeof(float) * b->Q);
    if (!rc) rc = balloc(b, (void **)&b->probe_d, sizeof(double) * 2 * n);
    if (!rc) rc = balloc(b, (void **)&b->delta_d, sizeof(float) * n);
    if (!rc) {
        std::vector<float> wq(b->w.begin(), b->w.end());
        if (cudaMemcpy(b->inst_d, b->inst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(b->wq_d, wq.data(), sizeof(float) * b->Q, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(b->counter, 0, 2 * sizeof(int)) != cudaSuccess ||
            cudaMemset(b->u_old, 0, fb * b->D) != cudaSuccess || cudaMemset(b->dn, 0, fb) != cudaSuccess)
            rc = fail(SCLBM_ERR_CUDA, "batch upload: %s", cudaGetErrorString(cudaGetLastError()));
    }
    if (!rc) rc = batch_plan(b);
    if (rc) {
        brelease(b);
        delete b;
        return rc;
    }
    *out = b;
    return SCLBM_OK;
}

int sclbm_batch_destroy(sclbm_batch *b) {
    if (!b) return SCLBM_OK;
    {
        DevGuard dg(b->device);
        cudaStreamSynchronize(b->st);
        brelease(b);
    }
    delete b;
    return SCLBM_OK;
}

int sclbm_batch_info(const sclbm_batch *b, int64_t *cells, int64_t *device_bytes) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (cells) *cells = b->Vtot;
    if (device_bytes) *device_bytes = b->device_bytes;
    return SCLBM_OK;
}

int sclbm_batch_set_density(sclbm_batch *b, int i, const double *n) {
    if (!b || !n || i < 0 || i >= b->n) return fail(SCLBM_ERR_ARG, "bad argument");
    DevGuard dg(b->device);
    CUDA_TRY(cudaStreamSynchronize(b->st));  // the observables kernels use dn as scratch
    const int64_t V = lattice_cells(b, i);
    std::vector<float> tmp(V);
    for (int64_t g = 0; g < V; g++) tmp[g] = (float)(n[g] - (double)b->inst[i].rho0);
    CUDA_TRY(cudaMemcpy((float *)b->dn + b->inst[i].base, tmp.data(), V * sizeof(float), cudaMemcpyHostToDevice));
    return SCLBM_OK;
}

int sclbm_batch_init_populations(sclbm_batch *b) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    DevGuard dg(b->device);
    const dim3 grid(b->gx, b->n);
    if (b->D == 2)
        k_batch_init<D2Q9><<<grid, BATCH_THREADS, 0, b->st>>>((float *)b->pop[b->cur], (const float *)b->dn, b->inst_d,
                                                             (int)b->Vtot, b->wq_d);
    else
        k_batch_init<D3Q19><<<grid, BATCH_THREADS, 0, b->st>>>((float *)b->pop[b->cur], (const float *)b->dn, b->inst_d,
                                                              (int)b->Vtot, b->wq_d);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(b->st));
    b->pop_set = true;
    return SCLBM_OK;
}

int sclbm_batch_init_lattice(sclbm_batch *b, int i) {
    if (!b || i < 0 || i >= b->n) return fail(SCLBM_ERR_ARG, "bad argument");
    if (!b->pop_set) return fail(SCLBM_ERR_STATE, "call sclbm_batch_init_populations first");
    if (b->home[i] >= 0) return fail(SCLBM_ERR_STATE, "lattice %d is retired", i);
    DevGuard dg(b->device);
    const dim3 grid(b->gx, 1);
    if (b->D == 2)
        k_batch_init<D2Q9><<<grid, BATCH_THREADS, 0, b->st>>>((float *)b->pop[b->cur], (const float *)b->dn,
                                                             b->inst_d + i, (int)b->Vtot, b->wq_d);
    else
        k_batch_init<D3Q19><<<grid, BATCH_THREADS, 0, b->st>>>((float *)b->pop[b->cur], (const float *)b->dn,
                                                              b->inst_d + i, (int)b->Vtot, b->wq_d);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(b->st));
    return SCLBM_OK;
}

int sclbm_batch_step(sclbm_batch *b, int64_t nsteps) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (!b->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    if (nsteps < 0) return fail(SCLBM_ERR_ARG, "nsteps < 0");
    DevGuard dg(b->device);
    int rc = batch_run(b, nsteps);
    if (!rc)
        for (int i = 0; i < b->n; i++)
            if (b->home[i] < 0) b->steps[i] += nsteps;
    return rc;
}

int sclbm_batch_step_timed(sclbm_batch *b, int64_t nsteps, double *ms) {
    if (!b || !ms) return fail(SCLBM_ERR_ARG, "bad argument");
    DevGuard dg(b->device);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    cudaEventRecord(e0, b->st);
    int rc = sclbm_batch_step(b, nsteps);
    cudaEventRecord(e1, b->st);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t;
    if (rc) return rc;
    CUDA_TRY(cudaGetLastError());
    return SCLBM_OK;
}

int sclbm_batch_check(sclbm_batch *b, double *u_conv, double *max_u, double *mass) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (!b->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(b->device);
    cudaError_t e = b->ops->batch_density(b->pop[b->cur], b->dn, b->psi, b->sp.data(), b->inst_d, b->n, (int)b->Vtot,
                                          b->gx, b->st);
    if (e == cudaSuccess)
        e = b->ops->batch_moments(b->pop[b->cur], b->dn, b->psi, b->u_old, b->sp.data(), b->inst_d, b->n,
                                  (int)b->Vtot, b->partials, b->gx, b->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "batch check: %s", cudaGetErrorString(e));
    std::vector<double> part((size_t)b->n * b->gx * BATCH_NV);
    CUDA_TRY(cudaMemcpyAsync(part.data(), b->partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    for (int i = 0; i < b->n; i++) {
        if (b->home[i] >= 0) continue;  // retired: keep the caller's last values
        double du = 0, mx = 0, m = 0;
        for (int k = 0; k < b->gx; k++) {
            const double *v = &part[((size_t)i * b->gx + k) * BATCH_NV];
            du += v[0];
            mx = std::max(mx, v[1]);
            m += v[2];
        }
        const double V = (double)lattice_cells(b, i);
        if (u_conv) u_conv[i] = du / V;
        if (max_u) max_u[i] = std::sqrt(mx / b->c2);
        if (mass) mass[i] = m;
    }
    return SCLBM_OK;
}

int sclbm_batch_set_active(sclbm_batch *b, const int *active) {
    if (!b || !active) return fail(SCLBM_ERR_ARG, "bad argument");
    DevGuard dg(b->device);
    CUDA_TRY(cudaStreamSynchronize(b->st));
    for (int i = 0; i < b->n; i++) {
        const bool on = active[i] != 0;
        if (!on && b->home[i] < 0) b->home[i] = b->cur;  // its state stays in this buffer
        if (on && b->home[i] >= 0) {
            // resuming: bring its state into the current buffer
            if (b->home[i] != b->cur) {
                const int64_t V = lattice_cells(b, i);
                for (int q = 0; q < b->Q; q++)
                    CUDA_TRY(cudaMemcpyAsync((float *)b->pop[b->cur] + (int64_t)q * b->Vtot + b->inst[i].base,
                                             (const float *)b->pop[b->home[i]] + (int64_t)q * b->Vtot +
                                                 b->inst[i].base,
                                             V * sizeof(float), cudaMemcpyDeviceToDevice, b->st));
            }
            b->home[i] = -1;
        }
        b->inst[i].active = on ? 1 : 0;
    }
    CUDA_TRY(cudaMemcpyAsync(b->inst_d, b->inst.data(), sizeof(BatchInst) * b->n, cudaMemcpyHostToDevice, b->st));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    return batch_plan(b);  // work items of the lattices still stepping
}

int sclbm_batch_get_density(sclbm_batch *b, int i, double *n) {
    if (!b || !n || i < 0 || i >= b->n) return fail(SCLBM_ERR_ARG, "bad argument");
    DevGuard dg(b->device);
    CUDA_TRY(cudaStreamSynchronize(b->st));
    const int64_t V = lattice_cells(b, i);
    const int buf = b->home[i] >= 0 ? b->home[i] : b->cur;
    std::vector<float> tmp(V);
    for (int64_t g = 0; g < V; g++) n[g] = b->inst[i].rho0;
    for (int i2 = 0; i2 < b->Q; i2++) {
        const int q = b->Q > 10 ? (int[]){0, 1, 10, 11, 12, 13, 14, 15, 16, 17, 18, 2, 3, 4, 5, 6, 7, 8, 9}[i2] : i2;
        CUDA_TRY(cudaMemcpy(tmp.data(), (const float *)b->pop[buf] + (int64_t)q * b->Vtot + b->inst[i].base,
                            V * sizeof(float), cudaMemcpyDeviceToHost));
        for (int64_t g = 0; g < V; g++) n[g] += (double)tmp[g];
    }
    return SCLBM_OK;
}

int sclbm_batch_restore_mass(sclbm_batch *b, const double *target, double *before) {
    if (!b || !target) return fail(SCLBM_ERR_ARG, "bad argument");
    if (!b->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(b->device);
    cudaError_t e = b->ops->batch_mass(b->pop[b->cur], b->inst_d, b->n, (int)b->Vtot, b->partials, b->gx, b->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "batch mass: %s", cudaGetErrorString(e));
    std::vector<double> part((size_t)b->n * b->gx * BATCH_NV);
    CUDA_TRY(cudaMemcpyAsync(part.data(), b->partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    std::vector<float> delta(b->n, 0.f);
    bool any = false;
    for (int i = 0; i < b->n; i++) {
        if (b->home[i] >= 0) continue;  // retired
        double m = 0;
        for (int k = 0; k < b->gx; k++) m += part[((size_t)i * b->gx + k) * BATCH_NV + 2];
        if (before) before[i] = m;
        if (std::isfinite(target[i]) && std::isfinite(m)) {
            delta[i] = (float)((target[i] - m) / (double)lattice_cells(b, i));
            any = any || delta[i] != 0.f;
        }
    }
    if (!any) return SCLBM_OK;
    CUDA_TRY(cudaMemcpyAsync(b->delta_d, delta.data(), sizeof(float) * b->n, cudaMemcpyHostToDevice, b->st));
    e = b->ops->batch_add_rest(b->pop[b->cur], b->inst_d, b->n, (int)b->Vtot, b->delta_d, b->gx, b->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "batch mass correction: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    return SCLBM_OK;
}

int sclbm_batch_set_tile_width(sclbm_batch *b, int tx) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (tx != 0 && !(b->D == 2 && tx == BATCH_TX_NARROW))
        return fail(SCLBM_ERR_ARG, "tile width %d (0, or %d for 2D batches)", tx, BATCH_TX_NARROW);
    if (tx == b->tx) return SCLBM_OK;
    DevGuard dg(b->device);
    b->tx = tx;
    return batch_plan(b);
}

int sclbm_batch_set_mass_compensation(sclbm_batch *b, int on) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (!on && !b->pairs)
        return fail(SCLBM_ERR_UNSUPPORTED, "the uncompensated step is built for 3D batches with paired halo loads only");
    b->exact_rest = on ? 1 : 0;
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;  // they hold the kernel
    return SCLBM_OK;
}

int sclbm_batch_set_probe_radius(sclbm_batch *b, int rad) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (rad < 0 || rad > 4) return fail(SCLBM_ERR_ARG, "probe radius %d (0 .. 4)", rad);
    b->probe_rad = rad;
    return SCLBM_OK;
}

int sclbm_batch_probe(sclbm_batch *b, double *n_in, double *n_out) {
    if (!b) return fail(SCLBM_ERR_ARG, "null handle");
    if (!b->pop_set) return fail(SCLBM_ERR_STATE, "populations are not initialized");
    DevGuard dg(b->device);
    cudaError_t e = b->ops->batch_probe(b->pop[b->cur], b->inst_d, b->n, (int)b->Vtot, b->probe_d, b->probe_rad,
                                        b->st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "batch probe: %s", cudaGetErrorString(e));
    std::vector<double> v((size_t)2 * b->n);
    CUDA_TRY(cudaMemcpyAsync(v.data(), b->probe_d, v.size() * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    for (int i = 0; i < b->n; i++) {
        if (b->home[i] >= 0) continue;  // retired: keep the caller's last values
        if (n_in) n_in[i] = v[2 * i];
        if (n_out) n_out[i] = v[2 * i + 1];
    }
    return SCLBM_OK;
}

int sclbm_batch_steps(const sclbm_batch *b, int64_t *steps) {
    if (!b || !steps) return fail(SCLBM_ERR_ARG, "bad argument");
    for (int i = 0; i < b->n; i++) steps[i] = b->steps[i];
    return SCLBM_OK;
}

}  // extern "C"

// ============================================================================
// One step with no device allocation (sclbm_step_noalloc).  The density+psi
// pass and the force+collide+stream pass need two scratch fields (density and
// psi, one value per cell) between them; here they live in a fixed array in the
// library's own device data, so the call allocates nothing.  The array is
// FP64-sized and split in two halves: the density at offset 0 and psi at
// offset SCLBM_NOALLOC_MAX_CELLS * 8 bytes (FP32 fields use the first half of
// each).  Every cell of both fields is written by the first pass before the
// second pass reads it, so nothing has to be cleared between calls.
static __device__ __align__(256) double g_noalloc_scratch[2 * (size_t)SCLBM_NOALLOC_MAX_CELLS];

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;

// The array's device address belongs to the CUDA context the library's module
// was loaded in.  A cudaDeviceReset (a new primary context) or a caller's own
// current context loads the module again, possibly elsewhere, so the cache
// holds the address together with the id of the context it was taken in
// (cuCtxGetId: unique for the life of the process, never reused).
struct NoallocSlot {
    unsigned long long ctx_id;
    void *addr;
};
NoallocSlot g_noalloc_slot[NOALLOC_MAX_DEVICES] = {};

using PfnCtxGetCurrent = CUresult (*)(CUcontext *);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long *);
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

// id of the context current on this thread (the runtime made the device's
// primary context current in DevGuard unless the caller has its own current)
int current_context_id(unsigned long long *id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        void *f1 = nullptr, *f2 = nullptr;
        const cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        const cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            cudaGetLastError();
            return fail(SCLBM_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId not available");
        }
        g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
        g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(f2);
    }
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return fail(SCLBM_ERR_CUDA, "no current CUDA context");
    if (g_ctx_get_id(c, id) != CUDA_SUCCESS) return fail(SCLBM_ERR_CUDA, "cuCtxGetId failed");
    return SCLBM_OK;
}

// device address of the scratch array in the current context of device dev
// (looked up once per device and context; the host-side symbol itself is not a
// device address)
int noalloc_scratch(int dev, void **out) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(SCLBM_ERR_ARG, "device %d beyond %d", dev, NOALLOC_MAX_DEVICES);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long id = 0;
    {
        const int rc = current_context_id(&id);
        if (rc) return rc;
    }
    NoallocSlot &slot = g_noalloc_slot[dev];
    if (!slot.addr || slot.ctx_id != id) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(SCLBM_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev, cudaGetErrorString(e));
        }
        slot.ctx_id = id;
        slot.addr = p;
    }
    *out = slot.addr;
    return SCLBM_OK;
}

}  // namespace

extern "C" int sclbm_step_noalloc(const sclbm_params *p, const void *pop_in, void *pop_out, void *stream) {
    g_err.clear();
    if (!p || !pop_in || !pop_out) return fail(SCLBM_ERR_ARG, "null argument");
    if (p->dim != 2 && p->dim != 3) return fail(SCLBM_ERR_UNSUPPORTED, "dimension %d (2 or 3 supported)", p->dim);
    if (!p->xi || !p->w || !p->e || !p->we) return fail(SCLBM_ERR_ARG, "null stencil table");
    const int *cx = compiled_xi(p->dim, p->q);
    if (!cx) return fail(SCLBM_ERR_UNSUPPORTED, "lattice D%dQ%d not built (D2Q9, D3Q19)", p->dim, p->q);
    for (int i = 0; i < p->q * p->dim; i++)
        if (p->xi[i] != cx[i]) return fail(SCLBM_ERR_UNSUPPORTED, "lattice velocities differ from D%dQ%d", p->dim, p->q);
    const int order = stencil_order(p->dim, p->e, p->qe);
    if (!order) return fail(SCLBM_ERR_UNSUPPORTED, "force stencil (%d vectors) is not E4/E6/E8", p->qe);
    int64_t V = 1;
    for (int d = 0; d < p->dim; d++) {
        if (p->sizes[d] < 2 || p->sizes[d] > (1 << 24))
            return fail(SCLBM_ERR_ARG, "size[%d] = %d out of range [2, 2^24]", d, p->sizes[d]);
        V *= p->sizes[d];
    }
    if (V > SCLBM_NOALLOC_MAX_CELLS)
        return fail(SCLBM_ERR_ARG, "lattice of %lld cells exceeds the %d-cell scratch of sclbm_step_noalloc "
                    "(use a handle from sclbm_create)", (long long)V, SCLBM_NOALLOC_MAX_CELLS);
    if (p->psi_kind < 0 || p->psi_kind > 2) return fail(SCLBM_ERR_ARG, "psi_kind %d", p->psi_kind);
    if (p->precision != SCLBM_FP64 && p->precision != SCLBM_FP32_SHIFTED)
        return fail(SCLBM_ERR_ARG, "precision %d", p->precision);
    if (!(p->c2 > 0)) return fail(SCLBM_ERR_ARG, "c2 must be > 0");
    const size_t rs = p->precision == SCLBM_FP32_SHIFTED ? 4 : 8;
    const size_t bytes = (size_t)V * p->q * rs;
    const char *a = (const char *)pop_in, *b = (const char *)pop_out;
    if (a < b + bytes && b < a + bytes) return fail(SCLBM_ERR_ARG, "pop_in and pop_out overlap");

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SCLBM_ERR_NODEVICE, "no CUDA device visible");
    }
    if (p->device < 0 || p->device >= ndev) return fail(SCLBM_ERR_ARG, "device %d of %d", p->device, ndev);
    int major = 0, sms = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, p->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
        cudaGetLastError();
        return fail(SCLBM_ERR_CUDA, "device attributes");
    }
    if (major < 10) return fail(SCLBM_ERR_NODEVICE, "device %d is sm_%dx; built for sm_103a", p->device, major);
    DevGuard dg(p->device);
    // an error the caller's own work left pending on this thread stays the
    // caller's: it is neither reported as this step's failure nor cleared
    {
        const cudaError_t pend = cudaPeekAtLastError();
        if (pend != cudaSuccess)
            return fail(SCLBM_ERR_CUDA, "a CUDA error was already pending before the step (left uncleared): %s",
                        cudaGetErrorString(pend));
    }
    void *scratch = nullptr;
    {
        int rc = noalloc_scratch(p->device, &scratch);
        if (rc) return rc;
    }
    // host-side configuration only: the same kernel set, launch parameters and
    // grids as a handle with these parameters (configure() touches no device memory)
    sclbm_sim s;
    s.device = p->device;
    s.D = p->dim;
    s.Q = p->q;
    s.QE = p->qe;
    s.order = order;
    s.V = V;
    for (int d = 0; d < s.D; d++) s.L[d] = p->sizes[d];
    s.fp32 = p->precision == SCLBM_FP32_SHIFTED;
    s.rs = rs;
    s.rho0 = s.fp32 ? p->rho0 : 0.0;
    s.c2 = p->c2;
    s.G = p->sc_g;
    s.psi_kind = p->psi_kind;
    s.literals = p->literals;
    s.sms = sms;
    s.path = SCLBM_PATH_TWO_PASS;
    s.w.assign(p->w, p->w + p->q);
    s.we.assign(p->we, p->we + p->qe);
    s.xi.assign(p->xi, p->xi + p->q * p->dim);
    s.e.assign(p->e, p->e + p->qe * p->dim);
    {
        int rc = configure(&s, p->collision, p->tau, p->mrt_s, p->coll_a, p->coll_b);
        if (rc) return rc;
    }
    void *dn = scratch;
    void *psi = (char *)scratch + (size_t)SCLBM_NOALLOC_MAX_CELLS * sizeof(double);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = s.ops->density(pop_in, dn, psi, s.sp.data(), s.dgrid, st);
    if (e == cudaSuccess) e = s.ops->fcs(pop_in, pop_out, dn, psi, s.sp.data(), s.fgrid, st);
    if (e != cudaSuccess) return fail(SCLBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    return SCLBM_OK;
}
