// Surrogate MLP for droplet warm starts: 5 -> 64 -> 64 -> 64 -> 1, SiLU,
// BF16 parameters and activations as GEMM operands, FP32 accumulation, Adam.
// The reference has no counterpart (it always starts from a tanh profile).
//
// One training step is three kernels (captured in CUDA graphs):
//   k_mlp_tile   every CTA draws 64 samples, runs forward and backward and
//                writes its partial gradient (and loss) to its own slot;
//   k_mlp_adam   one thread per parameter sums the CTA slots in a fixed order
//                (deterministic), applies Adam to the FP32 master copy and
//                writes the BF16 compute copies (and W^T for the backward GEMMs);
//   k_mlp_tick   advances the step counter the other two read.
// The 64-wide layers are warp-level tensor-core MMAs (mma.sync m16n8k16,
// bf16 x bf16 -> f32): warp w owns samples 16w..16w+15 of the CTA for the
// forward and back-propagation GEMMs, and rows 16w..16w+15 of the weight
// gradients (summed over the CTA's 64 samples) for dW = dZ^T H.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/sclbm.h"

namespace sclbm {
int set_error(int code, const char *msg);
void clear_error();
}  // namespace sclbm

namespace {

constexpr int H = 64, IN = 5;
constexpr int SPC = 64;          // samples per CTA
constexpr int WARPS = 4, NTHR = 32 * WARPS;
constexpr int LD = 72;           // padded row of the bf16 tiles (conflict-free fragment loads)
constexpr int LDZ = 68;          // padded row of the fp32 tiles
// parameter vector: W1 [64][5], b1, W2 [64][64], b2, W3 [64][64], b3, W4 [64], b4
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + H,
              NP = OFF_B4 + 1;
constexpr int PSTRIDE = (NP + 1 + 7) / 8 * 8;  // per-CTA partial slot: NP gradients + loss
constexpr int GRAPH_STEPS = 50;

struct Smem {
    __nv_bfloat16 W2[H * LD], W2T[H * LD], W3[H * LD], W3T[H * LD];
    __nv_bfloat16 h1[SPC * LD], h2[SPC * LD], h1T[H * LD], h2T[H * LD];
    __nv_bfloat16 dz[SPC * LD], dzT[H * LD];
    float z1[SPC * LDZ], z2[SPC * LDZ], z3[SPC * LDZ];
    float W1[H * IN], b1[H], b2[H], b3[H], W4[H], b4;
    float x[SPC * IN], t[SPC], dy[SPC], mask[SPC];
    float red[NTHR];
};

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = sigm(z);
    return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// C[16][64] = A[16][64] . B[64][64]^T for one warp: A rows (stride LD) hold
// the K = 64 reduction index contiguous, B rows (stride LD) are the 64 outputs
// with K contiguous.  acc[nt][0..3]: rows g, g, g+8, g+8; cols nt*8 + 2t, +1.
__device__ __forceinline__ void warp_gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float (&acc)[8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int i = 0; i < 4; i++) acc[nt][i] = 0.f;
#pragma unroll
    for (int kk = 0; kk < H; kk += 16) {
        const uint32_t a0 = ld32(A + g * LD + kk + 2 * t), a1 = ld32(A + (g + 8) * LD + kk + 2 * t);
        const uint32_t a2 = ld32(A + g * LD + kk + 2 * t + 8), a3 = ld32(A + (g + 8) * LD + kk + 2 * t + 8);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const __nv_bfloat16 *b = B + (nt * 8 + g) * LD + kk + 2 * t;
            mma16816(acc[nt], a0, a1, a2, a3, ld32(b), ld32(b + 8));
        }
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct TileArgs {
    const __nv_bfloat16 *wb;   // NP compute (bf16) parameters
    const __nv_bfloat16 *w2t;  // W2^T, W3^T [64][64]
    const __nv_bfloat16 *w3t;
    const float *x;            // data: n x 5 inputs, n targets
    const float *t;
    int64_t n;
    int64_t batch;             // samples of the step (loss scale)
    int random;                // 1: draw samples with the step counter; 0: samples cta*64 + s
    uint64_t seed;
    const int64_t *step;
    float *part;               // [CTA][PSTRIDE]
    float *y;                  // forward only: outputs (null when training)
};

// load the compute parameters of the layers into shared memory
__device__ void load_params(Smem &S, const TileArgs &a) {
    for (int e = threadIdx.x; e < H * H; e += NTHR) {
        const int r = e / H, c = e % H;
        S.W2[r * LD + c] = a.wb[OFF_W2 + e];
        S.W3[r * LD + c] = a.wb[OFF_W3 + e];
        S.W2T[r * LD + c] = a.w2t[e];
        S.W3T[r * LD + c] = a.w3t[e];
    }
    for (int e = threadIdx.x; e < H * IN; e += NTHR) S.W1[e] = __bfloat162float(a.wb[OFF_W1 + e]);
    for (int e = threadIdx.x; e < H; e += NTHR) {
        S.b1[e] = __bfloat162float(a.wb[OFF_B1 + e]);
        S.b2[e] = __bfloat162float(a.wb[OFF_B2 + e]);
        S.b3[e] = __bfloat162float(a.wb[OFF_B3 + e]);
        S.W4[e] = __bfloat162float(a.wb[OFF_W4 + e]);
    }
    if (threadIdx.x == 0) S.b4 = __bfloat162float(a.wb[OFF_B4]);
}

// z = acc + b; z -> zbuf (own rows), silu(z) -> h (row-major) and hT (transposed)
__device__ __forceinline__ void epilogue_fwd(const float (&acc)[8][4], const float *b, int s0, float *zbuf,
                                             __nv_bfloat16 *h, __nv_bfloat16 *hT) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int s = s0 + g + (i >= 2 ? 8 : 0), n = nt * 8 + 2 * t + (i & 1);
            const float z = acc[nt][i] + b[n];
            zbuf[s * LDZ + n] = z;
            if (h) {
                const __nv_bfloat16 v = __float2bfloat16_rn(silu(z));
                h[s * LD + n] = v;
                hT[n * LD + s] = v;
            }
        }
}

__global__ void __launch_bounds__(NTHR) k_mlp_tile(const TileArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int s0 = warp * 16;
    load_params(S, a);
    // the CTA's samples
    const int64_t step = a.step ? *a.step : 0;
    for (int s = tid; s < SPC; s += NTHR) {
        const int64_t j = (int64_t)blockIdx.x * SPC + s;
        int64_t idx = j;
        bool ok = j < a.batch && a.n > 0;
        if (a.random && ok) idx = (int64_t)(mix64(a.seed ^ mix64((uint64_t)step * 0x9E3779B97F4A7C15ull + (uint64_t)j)) %
                                            (uint64_t)a.n);
        ok = ok && idx < a.n;
        S.mask[s] = ok ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < IN; k++) S.x[s * IN + k] = ok ? a.x[idx * IN + k] : 0.f;
        S.t[s] = ok && a.t ? a.t[idx] : 0.f;
    }
    __syncthreads();
    // layer 1 (K = 5, CUDA cores)
    for (int e = tid; e < SPC * H; e += NTHR) {
        const int s = e / H, n = e % H;
        float z = S.b1[n];
#pragma unroll
        for (int k = 0; k < IN; k++) z = fmaf(S.W1[n * IN + k], S.x[s * IN + k], z);
        S.z1[s * LDZ + n] = z;
        const __nv_bfloat16 v = __float2bfloat16_rn(silu(z));
        S.h1[s * LD + n] = v;
        S.h1T[n * LD + s] = v;
    }
    __syncthreads();
    float acc[8][4];
    // layers 2 and 3 (tensor cores)
    warp_gemm(S.h1 + s0 * LD, S.W2, acc);
    epilogue_fwd(acc, S.b2, s0, S.z2, S.h2, S.h2T);
    __syncwarp();
    warp_gemm(S.h2 + s0 * LD, S.W3, acc);
    epilogue_fwd(acc, S.b3, s0, S.z3, nullptr, nullptr);
    __syncthreads();
    // layer 4 and the loss
    float l = 0.f;
    for (int s = tid; s < SPC; s += NTHR) {
        float y = S.b4;
        for (int k = 0; k < H; k++) y = fmaf(S.W4[k], silu(S.z3[s * LDZ + k]), y);
        const float d = (y - S.t[s]) * S.mask[s];
        if (a.y) {
            const int64_t j = (int64_t)blockIdx.x * SPC + s;
            if (j < a.batch) a.y[j] = y;
        }
        S.dy[s] = 2.f * d / (float)a.batch;
        l += d * d;
    }
    S.red[tid] = l;
    __syncthreads();
    if (a.y) return;  // forward only
    float *P = a.part + (size_t)blockIdx.x * PSTRIDE;
    if (tid == 0) {
        float s = 0.f, db = 0.f;
        for (int i = 0; i < NTHR; i++) s += S.red[i];
        for (int i = 0; i < SPC; i++) db += S.dy[i];
        P[NP] = s;
        P[OFF_B4] = db;
    }
    // dW4 = sum_s dy h3 (before z3 is overwritten by dz3)
    for (int k = tid; k < H; k += NTHR) {
        float g = 0.f;
        for (int s = 0; s < SPC; s++) g = fmaf(S.dy[s], silu(S.z3[s * LDZ + k]), g);
        P[OFF_W4 + k] = g;
    }
    __syncthreads();
    // dz3 = dy W4 silu'(z3)
    for (int e = tid; e < SPC * H; e += NTHR) {
        const int s = e / H, n = e % H;
        const float d = S.dy[s] * S.W4[n] * dsilu(S.z3[s * LDZ + n]);
        S.z3[s * LDZ + n] = d;
        const __nv_bfloat16 v = __float2bfloat16_rn(d);
        S.dz[s * LD + n] = v;
        S.dzT[n * LD + s] = v;
    }
    __syncthreads();
    // two hidden layers back: (dz of layer L+1 in dz/dzT and zL1, h of layer L)
    auto back = [&](float *zup, const __nv_bfloat16 *hT, const __nv_bfloat16 *WT, float *zlow, int offW,
                    int offB) {
        const int g = lane >> 2, t = lane & 3;
        // dW = dZ^T H over the CTA's samples: rows 16*warp.. of dW
        warp_gemm(S.dzT + s0 * LD, hT, acc);
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = s0 + g + (i >= 2 ? 8 : 0), c = nt * 8 + 2 * t + (i & 1);
                P[offW + r * H + c] = acc[nt][i];
            }
        for (int n = tid; n < H; n += NTHR) {
            float db = 0.f;
            for (int s = 0; s < SPC; s++) db += zup[s * LDZ + n];
            P[offB + n] = db;
        }
        // dH = dZ W (own samples), then dZ_low = dH silu'(z_low) in place of z_low
        warp_gemm(S.dz + s0 * LD, WT, acc);
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int s = s0 + g + (i >= 2 ? 8 : 0), k = nt * 8 + 2 * t + (i & 1);
                zlow[s * LDZ + k] = acc[nt][i] * dsilu(zlow[s * LDZ + k]);
            }
        __syncthreads();  // every reader of dz / dzT / zup is done
        for (int e = tid; e < SPC * H; e += NTHR) {
            const int s = e / H, k = e % H;
            const __nv_bfloat16 v = __float2bfloat16_rn(zlow[s * LDZ + k]);
            S.dz[s * LD + k] = v;
            S.dzT[k * LD + s] = v;
        }
        __syncthreads();
    };
    back(S.z3, S.h2T, S.W3T, S.z2, OFF_W3, OFF_B3);
    back(S.z2, S.h1T, S.W2T, S.z1, OFF_W2, OFF_B2);
    // layer 1: dW1 = dz1^T x, db1
    for (int e = tid; e < H * IN; e += NTHR) {
        const int n = e / IN, k = e % IN;
        float g = 0.f;
        for (int s = 0; s < SPC; s++) g = fmaf(S.z1[s * LDZ + n], S.x[s * IN + k], g);
        P[OFF_W1 + e] = g;
    }
    for (int n = tid; n < H; n += NTHR) {
        float db = 0.f;
        for (int s = 0; s < SPC; s++) db += S.z1[s * LDZ + n];
        P[OFF_B1 + n] = db;
    }
}

struct AdamArgs {
    float *w, *m, *v;          // FP32 master parameters and moments
    __nv_bfloat16 *wb, *w2t, *w3t;
    const float *part;
    int ncta;
    float lr, b1, b2, eps;
    const int64_t *step;
    float *loss_hist;          // [capacity] loss per step (mean over the batch)
    int64_t loss_cap;
    int64_t batch;
    float *grad_out;           // non-null: write the summed gradient and skip the update
};

__device__ __forceinline__ void write_compute_copy(const AdamArgs &a, int p, float w) {
    const __nv_bfloat16 v = __float2bfloat16_rn(w);
    a.wb[p] = v;
    if (p >= OFF_W2 && p < OFF_W2 + H * H) {
        const int e = p - OFF_W2;
        a.w2t[(e % H) * H + e / H] = v;
    } else if (p >= OFF_W3 && p < OFF_W3 + H * H) {
        const int e = p - OFF_W3;
        a.w3t[(e % H) * H + e / H] = v;
    }
}

__global__ void k_mlp_adam(const AdamArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        float s = 0.f;
        for (int c = 0; c < a.ncta; c++) s += a.part[(size_t)c * PSTRIDE + NP];
        const int64_t st = a.step ? *a.step : 0;
        if (a.grad_out) a.grad_out[NP] = s / (float)a.batch;
        else if (a.loss_hist && st < a.loss_cap) a.loss_hist[st] = s / (float)a.batch;
    }
    if (p >= NP) return;
    float g = 0.f;
    for (int c = 0; c < a.ncta; c++) g += a.part[(size_t)c * PSTRIDE + p];
    if (a.grad_out) {
        a.grad_out[p] = g;
        return;
    }
    const float t = (float)(*a.step + 1);
    const float m = a.b1 * a.m[p] + (1.f - a.b1) * g;
    const float v = a.b2 * a.v[p] + (1.f - a.b2) * g * g;
    a.m[p] = m;
    a.v[p] = v;
    const float mh = m / (1.f - powf(a.b1, t)), vh = v / (1.f - powf(a.b2, t));
    const float w = a.w[p] - a.lr * mh / (sqrtf(vh) + a.eps);
    a.w[p] = w;
    write_compute_copy(a, p, w);
}

__global__ void k_mlp_sync_copy(AdamArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NP) write_compute_copy(a, p, a.w[p]);
}

__global__ void k_mlp_tick(int64_t *step) { *step += 1; }

}  // namespace

struct sclbm_mlp {
    int device = 0;
    cudaStream_t st = nullptr;
    float *w = nullptr, *m = nullptr, *v = nullptr, *part = nullptr, *loss = nullptr, *grad = nullptr;
    __nv_bfloat16 *wb = nullptr, *w2t = nullptr, *w3t = nullptr;
    float *x = nullptr, *t = nullptr, *y = nullptr, *gx = nullptr, *gt = nullptr;
    int64_t n = 0, xcap = 0, tcap = 0, ycap = 0, gxcap = 0, gtcap = 0, loss_cap = 0, part_cta = 0;
    int64_t *step = nullptr;
    uint64_t seed = 0;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_batch = 0;
    float graph_lr = 0.f;
};

namespace {

int err(int code, const std::string &m) { return sclbm::set_error(code, m.c_str()); }

#define MLP_TRY(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return err(SCLBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct Guard {
    int prev = -1;
    explicit Guard(int d) {
        cudaGetDevice(&prev);
        if (prev != d) cudaSetDevice(d);
    }
    ~Guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int dalloc(void **p, size_t bytes) {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return err(SCLBM_ERR_NOMEM, "cudaMalloc(" + std::to_string(bytes) + ") failed");
    }
    return SCLBM_OK;
}

int ensure_part(sclbm_mlp *m, int64_t ncta) {
    if (ncta <= m->part_cta) return SCLBM_OK;
    if (m->graph) cudaGraphExecDestroy(m->graph), m->graph = nullptr;  // it holds the old slots
    if (m->part) cudaFree(m->part);
    m->part = nullptr;
    m->part_cta = 0;
    int rc = dalloc((void **)&m->part, (size_t)ncta * PSTRIDE * sizeof(float));
    if (!rc) m->part_cta = ncta;
    return rc;
}

int ensure_buf(float **p, int64_t *cap, int64_t n) {
    if (n <= *cap) return SCLBM_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    int rc = dalloc((void **)p, (size_t)n * sizeof(float));
    if (!rc) *cap = n;
    return rc;
}

constexpr size_t SMEM = sizeof(Smem);

int smem_attr() {
    static std::once_flag once[64];
    int dev = 0;
    cudaGetDevice(&dev);
    static cudaError_t res[64];
    if (dev < 0 || dev >= 64) return err(SCLBM_ERR_ARG, "device ordinal beyond 64");
    std::call_once(once[dev], [&] {
        res[dev] = cudaFuncSetAttribute(k_mlp_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    });
    if (res[dev] != cudaSuccess) return err(SCLBM_ERR_CUDA, std::string("shared memory attribute: ") +
                                                                cudaGetErrorString(res[dev]));
    return SCLBM_OK;
}

TileArgs tile_args(sclbm_mlp *m, const float *x, const float *t, int64_t n, int64_t batch, int random, float *y) {
    TileArgs a;
    a.wb = m->wb;
    a.w2t = m->w2t;
    a.w3t = m->w3t;
    a.x = x;
    a.t = t;
    a.n = n;
    a.batch = batch;
    a.random = random;
    a.seed = m->seed;
    a.step = m->step;
    a.part = m->part;
    a.y = y;
    return a;
}

AdamArgs adam_args(sclbm_mlp *m, int ncta, float lr, int64_t batch, float *grad_out) {
    AdamArgs a;
    a.w = m->w;
    a.m = m->m;
    a.v = m->v;
    a.wb = m->wb;
    a.w2t = m->w2t;
    a.w3t = m->w3t;
    a.part = m->part;
    a.ncta = ncta;
    a.lr = lr;
    a.b1 = 0.9f;
    a.b2 = 0.999f;
    a.eps = 1e-8f;
    a.step = m->step;
    a.loss_hist = m->loss;
    a.loss_cap = m->loss_cap;
    a.batch = batch;
    a.grad_out = grad_out;
    return a;
}

int enqueue_train_step(sclbm_mlp *m, int64_t batch, float lr) {
    const int ncta = (int)((batch + SPC - 1) / SPC);
    k_mlp_tile<<<ncta, NTHR, SMEM, m->st>>>(tile_args(m, m->x, m->t, m->n, batch, 1, nullptr));
    k_mlp_adam<<<(NP + 255) / 256, 256, 0, m->st>>>(adam_args(m, ncta, lr, batch, nullptr));
    k_mlp_tick<<<1, 1, 0, m->st>>>(m->step);
    MLP_TRY(cudaGetLastError());
    return SCLBM_OK;
}

}  // namespace

extern "C" {

int sclbm_mlp_param_count(int *count) {
    if (!count) return err(SCLBM_ERR_ARG, "null argument");
    *count = NP;
    return SCLBM_OK;
}

int sclbm_mlp_create(int device, uint64_t seed, sclbm_mlp **out) {
    sclbm::clear_error();
    if (!out) return err(SCLBM_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return err(SCLBM_ERR_NODEVICE, "no CUDA device visible");
    }
    if (device < 0 || device >= ndev) return err(SCLBM_ERR_ARG, "device out of range");
    Guard gd(device);
    int rc = smem_attr();
    if (rc) return rc;
    sclbm_mlp *m = new sclbm_mlp();
    m->device = device;
    m->seed = seed;
    if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete m;
        return err(SCLBM_ERR_CUDA, "stream create");
    }
    rc = dalloc((void **)&m->w, NP * sizeof(float));
    if (!rc) rc = dalloc((void **)&m->m, NP * sizeof(float));
    if (!rc) rc = dalloc((void **)&m->v, NP * sizeof(float));
    if (!rc) rc = dalloc((void **)&m->wb, NP * sizeof(__nv_bfloat16));
    if (!rc) rc = dalloc((void **)&m->w2t, H * H * sizeof(__nv_bfloat16));
    if (!rc) rc = dalloc((void **)&m->w3t, H * H * sizeof(__nv_bfloat16));
    if (!rc) rc = dalloc((void **)&m->step, sizeof(int64_t));
    if (!rc) rc = dalloc((void **)&m->grad, (NP + 1) * sizeof(float));
    if (rc) {
        sclbm_mlp_destroy(m);
        return rc;
    }
    // default initialisation: uniform in +-1/sqrt(fan_in) (weights and biases)
    std::vector<float> w(NP);
    uint64_t s = seed;
    auto uni = [&](float bound) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        const double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
        return (float)((2.0 * u - 1.0) * bound);
    };
    const float b1 = 1.f / std::sqrt((float)IN), bh = 1.f / std::sqrt((float)H);
    for (int i = 0; i < NP; i++) w[i] = uni(i < OFF_W2 ? b1 : bh);
    rc = sclbm_mlp_set_params(m, w.data());
    if (rc) {
        sclbm_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return SCLBM_OK;
}

int sclbm_mlp_destroy(sclbm_mlp *m) {
    if (!m) return SCLBM_OK;
    Guard gd(m->device);
    if (m->graph) cudaGraphExecDestroy(m->graph);
    for (void *p : {(void *)m->w, (void *)m->m, (void *)m->v, (void *)m->part, (void *)m->loss, (void *)m->grad,
                    (void *)m->wb, (void *)m->w2t, (void *)m->w3t, (void *)m->x, (void *)m->t, (void *)m->y,
                    (void *)m->gx, (void *)m->gt, (void *)m->step})
        if (p) cudaFree(p);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
    return SCLBM_OK;
}

int sclbm_mlp_set_params(sclbm_mlp *m, const float *w) {
    if (!m || !w) return err(SCLBM_ERR_ARG, "null argument");
    Guard gd(m->device);
    MLP_TRY(cudaMemcpyAsync(m->w, w, NP * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemsetAsync(m->m, 0, NP * sizeof(float), m->st));
    MLP_TRY(cudaMemsetAsync(m->v, 0, NP * sizeof(float), m->st));
    MLP_TRY(cudaMemsetAsync(m->step, 0, sizeof(int64_t), m->st));
    k_mlp_sync_copy<<<(NP + 255) / 256, 256, 0, m->st>>>(adam_args(m, 0, 0.f, 1, nullptr));
    MLP_TRY(cudaGetLastError());
    MLP_TRY(cudaStreamSynchronize(m->st));
    return SCLBM_OK;
}

int sclbm_mlp_get_params(sclbm_mlp *m, float *w) {
    if (!m || !w) return err(SCLBM_ERR_ARG, "null argument");
    Guard gd(m->device);
    MLP_TRY(cudaMemcpyAsync(w, m->w, NP * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    return SCLBM_OK;
}

int sclbm_mlp_set_data(sclbm_mlp *m, int64_t n, const float *x, const float *t) {
    if (!m || !x || !t || n < 1) return err(SCLBM_ERR_ARG, "bad argument");
    Guard gd(m->device);
    if (m->graph) cudaGraphExecDestroy(m->graph), m->graph = nullptr;  // it holds the old buffers
    int rc = ensure_buf(&m->x, &m->xcap, n * IN);
    if (!rc) rc = ensure_buf(&m->t, &m->tcap, n);
    if (rc) return rc;
    MLP_TRY(cudaMemcpyAsync(m->x, x, (size_t)n * IN * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->t, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    m->n = n;
    return SCLBM_OK;
}

int sclbm_mlp_train(sclbm_mlp *m, int64_t steps, int64_t batch, float lr, float *loss) {
    if (!m || steps < 0 || batch < 1 || !(lr > 0)) return err(SCLBM_ERR_ARG, "bad argument");
    if (m->n < 1) return err(SCLBM_ERR_STATE, "no training data (sclbm_mlp_set_data)");
    Guard gd(m->device);
    int rc = ensure_part(m, (batch + SPC - 1) / SPC);
    if (rc) return rc;
    int64_t start = 0;
    MLP_TRY(cudaMemcpyAsync(&start, m->step, sizeof(int64_t), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    if (start + steps > m->loss_cap) {
        float *old = m->loss;
        const int64_t cap = std::max<int64_t>(start + steps, 2 * m->loss_cap);
        float *nl = nullptr;
        rc = dalloc((void **)&nl, (size_t)cap * sizeof(float));
        if (rc) return rc;
        if (old) {
            MLP_TRY(cudaMemcpyAsync(nl, old, (size_t)m->loss_cap * sizeof(float), cudaMemcpyDeviceToDevice, m->st));
            MLP_TRY(cudaStreamSynchronize(m->st));
            cudaFree(old);
        }
        m->loss = nl;
        m->loss_cap = cap;
        if (m->graph) cudaGraphExecDestroy(m->graph), m->graph = nullptr;
    }
    if (m->graph && (m->graph_batch != batch || m->graph_lr != lr)) cudaGraphExecDestroy(m->graph), m->graph = nullptr;
    int64_t done = 0;
    if (steps >= GRAPH_STEPS) {
        if (!m->graph) {
            cudaGraph_t g;
            MLP_TRY(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
            int rc2 = SCLBM_OK;
            for (int i = 0; i < GRAPH_STEPS && !rc2; i++) rc2 = enqueue_train_step(m, batch, lr);
            cudaError_t ce = cudaStreamEndCapture(m->st, &g);
            if (rc2) return rc2;
            if (ce != cudaSuccess) return err(SCLBM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
            ce = cudaGraphInstantiate(&m->graph, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return err(SCLBM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
            m->graph_batch = batch;
            m->graph_lr = lr;
        }
        for (; done + GRAPH_STEPS <= steps; done += GRAPH_STEPS) MLP_TRY(cudaGraphLaunch(m->graph, m->st));
    }
    for (; done < steps; done++) {
        rc = enqueue_train_step(m, batch, lr);
        if (rc) return rc;
    }
    if (loss && steps > 0)
        MLP_TRY(cudaMemcpyAsync(loss, m->loss + start, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    return SCLBM_OK;
}

int sclbm_mlp_gradient(sclbm_mlp *m, int64_t n, const float *x, const float *t, float *grad, float *loss) {
    if (!m || !x || !t || !grad || n < 1) return err(SCLBM_ERR_ARG, "bad argument");
    Guard gd(m->device);
    int rc = ensure_buf(&m->gx, &m->gxcap, n * IN);
    if (!rc) rc = ensure_buf(&m->gt, &m->gtcap, n);
    if (rc) return rc;
    MLP_TRY(cudaMemcpyAsync(m->gx, x, (size_t)n * IN * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->gt, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->st));
    const int ncta = (int)((n + SPC - 1) / SPC);
    rc = ensure_part(m, ncta);
    if (rc) return rc;
    k_mlp_tile<<<ncta, NTHR, SMEM, m->st>>>(tile_args(m, m->gx, m->gt, n, n, 0, nullptr));
    k_mlp_adam<<<(NP + 255) / 256, 256, 0, m->st>>>(adam_args(m, ncta, 0.f, n, m->grad));
    MLP_TRY(cudaGetLastError());
    std::vector<float> g(NP + 1);
    MLP_TRY(cudaMemcpyAsync(g.data(), m->grad, (NP + 1) * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    std::memcpy(grad, g.data(), NP * sizeof(float));
    if (loss) *loss = g[NP];
    return SCLBM_OK;
}

int sclbm_mlp_predict(sclbm_mlp *m, int64_t n, const float *x, float *y) {
    if (!m || !x || !y || n < 1) return err(SCLBM_ERR_ARG, "bad argument");
    Guard gd(m->device);
    int64_t cap = m->ycap;
    int rc = ensure_buf(&m->y, &cap, n * (IN + 1));
    m->ycap = cap;
    if (rc) return rc;
    float *xd = m->y + n;  // inputs after the outputs
    MLP_TRY(cudaMemcpyAsync(xd, x, (size_t)n * IN * sizeof(float), cudaMemcpyHostToDevice, m->st));
    const int64_t ncta = (n + SPC - 1) / SPC;
    if (ncta > (int64_t)1 << 30) return err(SCLBM_ERR_ARG, "too many samples");
    k_mlp_tile<<<(unsigned)ncta, NTHR, SMEM, m->st>>>(tile_args(m, xd, nullptr, n, n, 0, m->y));
    MLP_TRY(cudaGetLastError());
    MLP_TRY(cudaMemcpyAsync(y, m->y, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    return SCLBM_OK;
}

}  // extern "C"
