// Per-patch MLP (32 -> 128 -> 128 -> 128 -> 128 -> 3, ReLU) with BF16 weights and
// FP32 accumulation: inference, backward and Adam, all hand-written kernels.
//
// It predicts a patch's converged radiosity from its geometry, reflectance,
// emission and first-shot direct light; the prediction only seeds the gathering
// solve (rad_gather_solve's guess), which still iterates to the same tolerance.
//
// Parameters: FP32 master copy (W_l row-major [out][in], then b_l) for Adam, and a
// BF16 copy of the weights used by the forward and backward passes.  Activations
// and gradients are FP32.  Layers process tiles of kRows patches per CTA; the
// BF16 weights are staged transposed in shared memory so threads (one per output
// channel) read conflict-free.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "radiosity.h"
#include "rad_internal.cuh"

namespace {

using rad::launch_gemm_tc;
using rad::TcEpilogue;

constexpr int kIn = 32, kHid = 128, kOut = 3, kLayers = 5;
constexpr int kRows = 32;  // patches per CTA tile
const int kDims[kLayers + 1] = {kIn, kHid, kHid, kHid, kHid, kOut};

// Y[r][o] = act(b[o] + sum_k X[r][k] W[o][k]) for a tile of kRows rows.
__global__ void __launch_bounds__(128) k_fwd(const float* __restrict__ X, uint32_t P, int in, int out,
                                             const __nv_bfloat16* __restrict__ W, const float* __restrict__ b,
                                             float* __restrict__ Y, int relu) {
    __shared__ __nv_bfloat16 Wt[kHid * kHid];  // [k][o]
    __shared__ float xs[kRows][kHid];
    for (int e = threadIdx.x; e < in * out; e += blockDim.x) {
        const int o = e / in, k = e % in;
        Wt[k * out + o] = W[e];
    }
    const uint32_t r0 = blockIdx.x * kRows;
    for (int e = threadIdx.x; e < kRows * in; e += blockDim.x) {
        const int r = e / in, k = e % in;
        xs[r][k] = (r0 + r < P) ? X[(size_t)(r0 + r) * in + k] : 0.f;
    }
    __syncthreads();
    const int o = threadIdx.x;
    if (o >= out) return;
    const float bo = b[o];
    for (int r = 0; r < kRows; r++) {
        if (r0 + r >= P) break;
        float acc = bo;
        for (int k = 0; k < in; k++) acc = fmaf(xs[r][k], __bfloat162float(Wt[k * out + o]), acc);
        if (relu) acc = fmaxf(acc, 0.f);
        Y[(size_t)(r0 + r) * out + o] = acc;
    }
}

// dZ = dY o relu'(Y), in place.
__global__ void k_relu_grad(float* __restrict__ dY, const float* __restrict__ Y, size_t total) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        if (!(Y[e] > 0.f)) dY[e] = 0.f;
}

// dX[r][k] = sum_o dZ[r][o] W[o][k] for a tile of kRows rows (W staged in shared memory).
__global__ void __launch_bounds__(128) k_bwd_dx(const float* __restrict__ dZ, uint32_t P, int in, int out,
                                                const __nv_bfloat16* __restrict__ W, float* __restrict__ dX) {
    __shared__ __nv_bfloat16 Ws[kHid * kHid];
    __shared__ float zs[kRows][kHid];
    for (int e = threadIdx.x; e < in * out; e += blockDim.x) Ws[e] = W[e];
    const uint32_t r0 = blockIdx.x * kRows;
    for (int e = threadIdx.x; e < kRows * out; e += blockDim.x) {
        const int r = e / out, o = e % out;
        zs[r][o] = (r0 + r < P) ? dZ[(size_t)(r0 + r) * out + o] : 0.f;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < in; k += blockDim.x)
        for (int r = 0; r < kRows; r++) {
            if (r0 + r >= P) break;
            float acc = 0.f;
            for (int o = 0; o < out; o++) acc = fmaf(zs[r][o], __bfloat162float(Ws[o * in + k]), acc);
            dX[(size_t)(r0 + r) * in + k] = acc;
        }
}

// dW[o][k] += sum_r dZ[r][o] X[r][k] and db[o] += sum_r dZ[r][o] over one chunk of rows.
__global__ void __launch_bounds__(128) k_bwd_dw(const float* __restrict__ dZ, const float* __restrict__ X, uint32_t P,
                                                int in, int out, uint32_t chunk, float* __restrict__ dW,
                                                float* __restrict__ db) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= in * out) return;
    const int o = e / in, k = e % in;
    const uint32_t r0 = blockIdx.y * chunk, r1 = min(P, r0 + chunk);
    float acc = 0.f, accb = 0.f;
    for (uint32_t r = r0; r < r1; r++) {
        const float z = dZ[(size_t)r * out + o];
        acc = fmaf(z, X[(size_t)r * in + k], acc);
        accb += z;
    }
    atomicAdd(&dW[e], acc);
    if (k == 0) atomicAdd(&db[o], accb);
}

// MSE loss on the final layer: dY = 2 (pred - target) / (P * kOut); loss partials.
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ tgt, uint32_t P, float* __restrict__ dY,
                      double* loss) {
    double part = 0;
    const size_t total = (size_t)P * kOut;
    const float scale = 2.0f / (float)total;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const float d = pred[e] - tgt[e];
        dY[e] = scale * d;
        part += (double)d * (double)d;
    }
    __shared__ double red[256];
    red[threadIdx.x] = part;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// Adam on the FP32 master copy, then refresh the BF16 weights.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       uint32_t n, float lr, float b1, float b2, float eps, float bc1, float bc2,
                       __nv_bfloat16* __restrict__ p16) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float upd = lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        const float np = p[i] - upd;
        p[i] = np;
        p16[i] = __float2bfloat16_rn(np);
    }
}

// Adam with the step count read on the device (ctr[0], already advanced for this step), for
// the captured training step of the tensor-core engine.
__global__ void k_adam_dev(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, uint32_t n, float lr, float b1, float b2, float eps,
                           const uint32_t* __restrict__ ctr, __nv_bfloat16* __restrict__ p16) {
    const float step = (float)ctr[0];
    const float bc1 = 1.f - powf(b1, step), bc2 = 1.f - powf(b2, step);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float np = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        p[i] = np;
        p16[i] = __float2bfloat16_rn(np);
    }
}

// Step counters of a captured training step: ctr[0] = Adam steps, ctr[1] = batch within the
// epoch's full batches (wraps after `full`).
__global__ void k_step_begin(uint32_t* ctr) { ctr[0] += 1; }
__global__ void k_step_end(uint32_t* ctr, uint32_t full) { ctr[1] = ctr[1] + 1 >= full ? 0 : ctr[1] + 1; }

__global__ void k_to_bf16(const float* __restrict__ p, uint32_t n, __nv_bfloat16* __restrict__ p16) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p16[i] = __float2bfloat16_rn(p[i]);
}

struct Offsets {
    size_t w[kLayers], b[kLayers], total;
};

Offsets offsets() {
    Offsets o{};
    size_t at = 0;
    for (int l = 0; l < kLayers; l++) {
        o.w[l] = at;
        at += (size_t)kDims[l + 1] * kDims[l];
        o.b[l] = at;
        at += (size_t)kDims[l + 1];
    }
    o.total = at;
    return o;
}

}  // namespace

struct rad_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    Offsets off{};
    float* p = nullptr;            // FP32 master
    __nv_bfloat16* p16 = nullptr;  // BF16 copy (weights and biases; biases are read as FP32 from p)
    float *g = nullptr, *m = nullptr, *v = nullptr;
    uint32_t step = 0;
    // activations for a batch
    uint32_t cap = 0;
    float* act[kLayers + 1] = {};
    float* dact[kLayers + 1] = {};
    float* tgt = nullptr;
    double* loss = nullptr;
    // tensor-core engine (tcgen05 BF16 GEMMs, FP32 accumulation; see tc_forward / tc_backward)
    bool tc = true;
    uint32_t tc_cap = 0;                       // rows the tc buffers hold (a multiple of 64)
    __nv_bfloat16* w16[kLayers] = {};          // W_l, [NRout][Kin] (zero padded)
    __nv_bfloat16* wt16[kLayers] = {};         // W_l^T, [NRin][Kout] (zero padded)
    __nv_bfloat16* ar[kLayers] = {};           // layer inputs, row-major [P][Kin]
    __nv_bfloat16* ac[kLayers] = {};           // layer inputs, column-major [in][cap]
    __nv_bfloat16* zr[kLayers] = {};           // output gradients dZ_l, row-major [P][Kout]
    __nv_bfloat16* zc[kLayers] = {};           // dZ_l, column-major [out][cap]
    float* y = nullptr;                        // network output, [P][3]
    float* part = nullptr;                     // split-K partial sums of the weight gradients
    uint32_t* ctr = nullptr;                   // device step counters of the captured training step
};

// ---- tensor-core engine --------------------------------------------------------------------
// Each layer is a tcgen05 GEMM C = A Bt^T of k_gemm_tc (128-row tiles, TMA-fed, FP32 in
// TMEM) with the layer's work fused into the epilogue:
//   forward  Z_l = A_l W_l^T: A_l row-major BF16 [P][Kin], Bt = W_l [out][Kin]; epilogue
//            bias + ReLU, BF16 written row-major (next A) and column-major (dW operand);
//            the last layer writes FP32 Y = Z + b;
//   dW_l     = dZ_l^T A_l: A = dZ_l column-major [out][P], Bt = A_l column-major [in][P],
//            K = P split over CTAs (k_tc_finalize adds the splits in order);
//   dX_l     = dZ_l W_l: A = dZ_l row-major [P][Kout], Bt = W_l^T [in][Kout]; epilogue
//            masks with A_l > 0 (the ReLU of the layer below) and writes dZ_{l-1} in BF16,
//            row- and column-major.
// Activations and output gradients are BF16 (tensor-core operands), sums FP32; the FP32
// master weights, biases, their gradients and Adam stay as in the CUDA-core engine.
const uint32_t kKin[kLayers] = {64, 128, 128, 128, 128};      // in, padded to the 64-wide K block
const uint32_t kKout[kLayers] = {128, 128, 128, 128, 64};     // out, padded likewise
const uint32_t kNRout[kLayers] = {128, 128, 128, 128, 16};    // GEMM widths of out
const uint32_t kNRin[kLayers] = {32, 128, 128, 128, 128};     // GEMM widths of in

__device__ __forceinline__ uint32_t pad64(uint32_t x) { return (x + 63u) & ~63u; }

// W_l -> w16 [NRout][Kin] and wt16 [NRin][Kout] (BF16, zero padded); layer = blockIdx.y.
struct TcWeights {
    __nv_bfloat16* w16[kLayers];
    __nv_bfloat16* wt16[kLayers];
    uint32_t wo[kLayers];
};
__global__ void k_tc_weights(const float* __restrict__ p, TcWeights tw) {
    const int l = blockIdx.y;
    const int in = l == 0 ? kIn : kHid, out = l == kLayers - 1 ? kOut : kHid;
    const uint32_t kin = l == 0 ? 64u : 128u, kout = l == kLayers - 1 ? 64u : 128u;
    const uint32_t nrout = l == kLayers - 1 ? 16u : 128u, nrin = l == 0 ? 32u : 128u;
    const float* W = p + tw.wo[l];
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < 128u * 128u; e += gridDim.x * blockDim.x) {
        if (e < nrout * kin) {
            const uint32_t o = e / kin, k = e % kin;
            tw.w16[l][e] = __float2bfloat16_rn((int)o < out && (int)k < in ? W[o * in + k] : 0.f);
        }
        if (e < nrin * kout) {
            const uint32_t i = e / kout, o = e % kout;
            tw.wt16[l][e] = __float2bfloat16_rn((int)o < out && (int)i < in ? W[o * in + i] : 0.f);
        }
    }
}

// One row of X (32 FP32) -> A_0: BF16 row-major [r][0..32) (columns 32..63 stay zero) as four
// 16-byte stores, and column-major [k][r] (consecutive rows in consecutive lanes: coalesced).
__device__ __forceinline__ void tc_input_row(const float* __restrict__ x, uint32_t r, uint32_t K,
                                             __nv_bfloat16* __restrict__ ar, __nv_bfloat16* __restrict__ ac) {
    const float4* x4 = reinterpret_cast<const float4*>(x);
    uint32_t packed[16];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const float4 f = x4[q];
        const __nv_bfloat162 h0 = __floats2bfloat162_rn(f.x, f.y), h1 = __floats2bfloat162_rn(f.z, f.w);
        packed[2 * q] = *reinterpret_cast<const uint32_t*>(&h0);
        packed[2 * q + 1] = *reinterpret_cast<const uint32_t*>(&h1);
        ac[(size_t)(4 * q) * K + r] = h0.x;
        ac[(size_t)(4 * q + 1) * K + r] = h0.y;
        ac[(size_t)(4 * q + 2) * K + r] = h1.x;
        ac[(size_t)(4 * q + 3) * K + r] = h1.y;
    }
    uint4* dst = reinterpret_cast<uint4*>(ar + (size_t)r * 64);
#pragma unroll
    for (int q = 0; q < 4; q++) dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
}

// The batch ctr[1] of a data set on the device: rows [ctr[1] * P, +P) of X -> A_0 (as
// k_tc_input) and of T -> tgt; thread per row.
__global__ void k_tc_batch(const float* __restrict__ X, const float* __restrict__ T, uint32_t P, uint32_t K,
                           const uint32_t* __restrict__ ctr, __nv_bfloat16* __restrict__ ar,
                           __nv_bfloat16* __restrict__ ac, float* __restrict__ tgt) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P) return;
    const size_t src = (size_t)ctr[1] * P + r;
    tc_input_row(X + src * kIn, r, K, ar, ac);
#pragma unroll
    for (int k = 0; k < kOut; k++) tgt[(size_t)r * kOut + k] = T[src * kOut + k];
}

// X (P x 32 FP32) -> A_0 row-major [P][64] and column-major [32][K] in BF16 (K = pad64(P),
// the row pitch of every column-major buffer for this batch); thread per row.
__global__ void k_tc_input(const float* __restrict__ X, uint32_t P, uint32_t K, __nv_bfloat16* __restrict__ ar,
                           __nv_bfloat16* __restrict__ ac) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < P) tc_input_row(X + (size_t)r * kIn, r, K, ar, ac);
}

// MSE: dY = 2 (Y - T) / (3P) in BF16 (row-major [P][64], column-major [3][K]); loss sum.
__global__ void k_tc_mse(const float* __restrict__ Y, const float* __restrict__ T, uint32_t P, uint32_t K,
                         __nv_bfloat16* __restrict__ zr, __nv_bfloat16* __restrict__ zc, double* loss) {
    double part = 0;
    const float scale = 2.0f / (float)((size_t)P * kOut);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < P * (uint32_t)kOut; e += gridDim.x * blockDim.x) {
        const uint32_t r = e / kOut, c = e % kOut;
        const float d = Y[e] - T[e];
        const __nv_bfloat16 h = __float2bfloat16_rn(scale * d);
        zr[(size_t)r * 64 + c] = h;
        zc[(size_t)c * K + r] = h;
        part += (double)d * (double)d;
    }
    __shared__ double red[256];
    red[threadIdx.x] = part;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// db_l[o] = sum over rows of dZ_l[r][o] (column-major BF16, pitch K), one CTA per output:
// 8 rows per 16-byte load, four loads in flight per thread (K is a multiple of 64 and the
// columns [P, K) are zero).
__global__ void __launch_bounds__(256) k_tc_bias_grad(const __nv_bfloat16* __restrict__ zc, uint32_t K,
                                                      float* __restrict__ db) {
    const uint32_t o = blockIdx.x;
    const uint4* src = reinterpret_cast<const uint4*>(zc + (size_t)o * K);
    const uint32_t nv = K / 8u;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint32_t v0 = threadIdx.x; v0 < nv; v0 += 4u * blockDim.x) {
        uint4 q[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint32_t v = v0 + (uint32_t)u * blockDim.x;
            q[u] = v < nv ? src[v] : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q[u]);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float2 f = __bfloat1622float2(h[j]);
                acc[u] += f.x + f.y;
            }
        }
    }
    __shared__ float red[256];
    red[threadIdx.x] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[o] = red[0];
}

static void tc_free_acts(rad_mlp* m) {
    for (int l = 0; l < kLayers; l++) {
        cudaFree(m->ar[l]); cudaFree(m->ac[l]); cudaFree(m->zr[l]); cudaFree(m->zc[l]);
        m->ar[l] = m->ac[l] = m->zr[l] = m->zc[l] = nullptr;
    }
    cudaFree(m->y);
    cudaFree(m->part);
    m->y = nullptr;
    m->part = nullptr;
    m->tc_cap = 0;
}

constexpr uint32_t kDwSplits = 148;  // K splits of a weight-gradient GEMM (at most; about one per SM)
constexpr uint32_t kMinRows = 128;  // GEMM operands hold at least one full 128-row tile

// Activation buffers for batches of up to P rows (at least kMinRows, a multiple of 64).
static int tc_ensure(rad_mlp* m, uint32_t P) {
    const uint32_t cap = std::max(kMinRows, (P + 63u) & ~63u);
    if (m->tc_cap >= cap) return RAD_OK;
    tc_free_acts(m);
    bool ok = true;
    for (int l = 0; l < kLayers && ok; l++) {
        ok = cudaMalloc(&m->ar[l], 2 * (size_t)cap * kKin[l]) == cudaSuccess &&
             cudaMalloc(&m->ac[l], 2 * (size_t)kNRin[l] * cap) == cudaSuccess &&
             cudaMalloc(&m->zr[l], 2 * (size_t)cap * kKout[l]) == cudaSuccess &&
             cudaMalloc(&m->zc[l], 2 * (size_t)kMinRows * cap) == cudaSuccess;
        // padding never written by the kernels stays zero (columns past `in` / `out` of the
        // row-major buffers, rows past `out` of the column-major output gradients)
        ok = ok && cudaMemset(m->ar[l], 0, 2 * (size_t)cap * kKin[l]) == cudaSuccess &&
             cudaMemset(m->ac[l], 0, 2 * (size_t)kNRin[l] * cap) == cudaSuccess &&
             cudaMemset(m->zr[l], 0, 2 * (size_t)cap * kKout[l]) == cudaSuccess &&
             cudaMemset(m->zc[l], 0, 2 * (size_t)kMinRows * cap) == cudaSuccess;
    }
    ok = ok && cudaMalloc(&m->y, 4 * (size_t)cap * kOut) == cudaSuccess &&
         cudaMalloc(&m->part, 4 * (size_t)kDwSplits * kHid * kHid) == cudaSuccess;
    if (!ok) {
        tc_free_acts(m);
        return RAD_E_NOMEM;
    }
    m->tc_cap = cap;
    return RAD_OK;
}

// BF16 copies of the weights for the tensor-core engine (after any change of the master).
static void tc_refresh(rad_mlp* m) {
    TcWeights tw{};
    for (int l = 0; l < kLayers; l++) {
        tw.w16[l] = m->w16[l];
        tw.wt16[l] = m->wt16[l];
        tw.wo[l] = (uint32_t)m->off.w[l];
    }
    k_tc_weights<<<dim3(16, kLayers), 256, 0, m->stream>>>(m->p, tw);
}

// Forward pass of the P rows staged by tc_stage (m->ar[0], m->ac[0]); output in m->y.
static int tc_forward(rad_mlp* m, uint32_t P) {
    const uint32_t K = (P + 63u) & ~63u;  // pitch of the column-major activations
    for (int l = 0; l < kLayers; l++) {
        TcEpilogue ep{};
        ep.n = P;
        ep.R = (uint32_t)kDims[l + 1];
        ep.bias = m->p + m->off.b[l];
        if (l < kLayers - 1) {
            ep.mode = 2;
            ep.out16r = m->ar[l + 1];
            ep.ldr = kKin[l + 1];
            ep.out16 = m->ac[l + 1];
            ep.ld16 = K;
        } else {
            ep.mode = 3;
            ep.out = m->y;
        }
        if (launch_gemm_tc(m->ar[l], std::max(P, kMinRows), kKin[l], m->w16[l], kNRout[l], ep, m->stream) != 0)
            return RAD_E_CUDA;
    }
    return RAD_OK;
}

// Loss and every parameter gradient (into m->g) of the batch whose forward pass ran.
static int tc_backward(rad_mlp* m, uint32_t P) {
    const uint32_t K = (P + 63u) & ~63u;  // rows of the weight-gradient GEMMs (their K)
    cudaMemsetAsync(m->loss, 0, sizeof(double), m->stream);
    if (K > P)  // the weight-gradient GEMMs run K over pad64(P) columns: the tail must be zero
        cudaMemset2DAsync(m->zc[kLayers - 1] + P, 2 * (size_t)K, 0, 2 * (size_t)(K - P), kOut, m->stream);
    k_tc_mse<<<152, 256, 0, m->stream>>>(m->y, m->tgt, P, K, m->zr[kLayers - 1], m->zc[kLayers - 1], m->loss);
    const uint32_t splits = std::min<uint32_t>(kDwSplits, K / 64u);
    for (int l = kLayers - 1; l >= 0; l--) {
        const uint32_t in = (uint32_t)kDims[l], out = (uint32_t)kDims[l + 1];
        TcEpilogue ep{};  // dW_l = dZ_l^T A_l, K = rows (split)
        ep.mode = 5;
        ep.n = out;
        ep.R = in;
        ep.out = m->g + m->off.w[l];
        ep.ldr = in;
        ep.partial = splits > 1 ? m->part : nullptr;
        ep.ksplit = splits;
        if (launch_gemm_tc(m->zc[l], kMinRows, K, m->ac[l], kNRin[l], ep, m->stream) != 0) return RAD_E_CUDA;
        k_tc_bias_grad<<<out, 256, 0, m->stream>>>(m->zc[l], K, m->g + m->off.b[l]);
        if (l > 0) {  // dZ_{l-1} = (dZ_l W_l) o [A_l > 0]
            TcEpilogue ex{};
            ex.mode = 4;
            ex.n = P;
            ex.R = in;
            ex.mask = m->ar[l];
            ex.ldm = kKin[l];
            ex.out16r = m->zr[l - 1];
            ex.ldr = kKout[l - 1];
            ex.out16 = m->zc[l - 1];
            ex.ld16 = K;
            if (K > P)
                cudaMemset2DAsync(m->zc[l - 1] + P, 2 * (size_t)K, 0, 2 * (size_t)(K - P), in, m->stream);
            if (launch_gemm_tc(m->zr[l], std::max(P, kMinRows), kKout[l], m->wt16[l], kNRin[l], ex, m->stream) != 0)
                return RAD_E_CUDA;
        }
    }
    return RAD_OK;
}

// Stages P rows of X (device) for the tensor-core passes and zeroes the columns [P, K) of the
// column-major activations (the weight-gradient GEMMs read them; an earlier, larger batch
// may have left values there).
static void tc_stage(rad_mlp* m, const float* dX, uint32_t P) {
    const uint32_t K = (P + 63u) & ~63u;
    if (K > P)
        for (int l = 0; l < kLayers; l++)
            cudaMemset2DAsync(m->ac[l] + P, 2 * (size_t)K, 0, 2 * (size_t)(K - P), kNRin[l], m->stream);
    k_tc_input<<<(P + 127) / 128, 128, 0, m->stream>>>(dX, P, K, m->ar[0], m->ac[0]);
}

static int mlp_ensure(rad_mlp* m, uint32_t P) {
    if (m->cap >= P) return RAD_OK;
    for (int l = 0; l <= kLayers; l++) {
        cudaFree(m->act[l]);
        cudaFree(m->dact[l]);
        if (cudaMalloc(&m->act[l], sizeof(float) * (size_t)P * kDims[l]) != cudaSuccess) return RAD_E_NOMEM;
        if (cudaMalloc(&m->dact[l], sizeof(float) * (size_t)P * kDims[l]) != cudaSuccess) return RAD_E_NOMEM;
    }
    cudaFree(m->tgt);
    if (cudaMalloc(&m->tgt, sizeof(float) * (size_t)P * kOut) != cudaSuccess) return RAD_E_NOMEM;
    m->cap = P;
    return RAD_OK;
}

static void mlp_forward(rad_mlp* m, uint32_t P) {
    const unsigned blocks = (P + kRows - 1) / kRows;
    for (int l = 0; l < kLayers; l++)
        k_fwd<<<blocks, 128, 0, m->stream>>>(m->act[l], P, kDims[l], kDims[l + 1], m->p16 + m->off.w[l],
                                             m->p + m->off.b[l], m->act[l + 1], l < kLayers - 1);
}

// Loss + gradients of the batch already in act[0] / tgt; gradients land in m->g.
static void mlp_backward(rad_mlp* m, uint32_t P) {
    const unsigned blocks = (P + kRows - 1) / kRows;
    cudaMemsetAsync(m->g, 0, sizeof(float) * m->off.total, m->stream);
    cudaMemsetAsync(m->loss, 0, sizeof(double), m->stream);
    k_mse<<<152, 256, 0, m->stream>>>(m->act[kLayers], m->tgt, P, m->dact[kLayers], m->loss);
    const uint32_t chunk = 512;
    for (int l = kLayers - 1; l >= 0; l--) {
        const int in = kDims[l], out = kDims[l + 1];
        if (l < kLayers - 1)
            k_relu_grad<<<152, 256, 0, m->stream>>>(m->dact[l + 1], m->act[l + 1], (size_t)P * out);
        dim3 g((in * out + 127) / 128, (P + chunk - 1) / chunk);
        k_bwd_dw<<<g, 128, 0, m->stream>>>(m->dact[l + 1], m->act[l], P, in, out, chunk, m->g + m->off.w[l],
                                           m->g + m->off.b[l]);
        if (l > 0)
            k_bwd_dx<<<blocks, 128, 0, m->stream>>>(m->dact[l + 1], P, in, out, m->p16 + m->off.w[l], m->dact[l]);
    }
}

namespace rad {
void mlp_forward_device(const rad_mlp* m, const float* X, uint32_t P, float* act0, float* act1, float* Y,
                        cudaStream_t s) {
    const unsigned blocks = (P + kRows - 1) / kRows;
    const float* in = X;
    for (int l = 0; l < kLayers; l++) {
        float* out = l == kLayers - 1 ? Y : ((l & 1) ? act1 : act0);
        k_fwd<<<blocks, 128, 0, s>>>(in, P, kDims[l], kDims[l + 1], m->p16 + m->off.w[l], m->p + m->off.b[l], out,
                                     l < kLayers - 1);
        in = out;
    }
}
}  // namespace rad

extern "C" {

int rad_mlp_create(int device, uint64_t seed, rad_mlp** out) {
    if (!out) return RAD_E_INVALID;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess || rad::dense_init() != cudaSuccess) return RAD_E_CUDA;
    rad_mlp* m = new rad_mlp();
    m->device = device;
    m->off = offsets();
    const size_t n = m->off.total;
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&m->p, 4 * n) != cudaSuccess || cudaMalloc(&m->p16, 2 * n) != cudaSuccess ||
        cudaMalloc(&m->g, 4 * n) != cudaSuccess || cudaMalloc(&m->m, 4 * n) != cudaSuccess ||
        cudaMalloc(&m->v, 4 * n) != cudaSuccess || cudaMalloc(&m->loss, 8) != cudaSuccess ||
        cudaMalloc(&m->ctr, 8) != cudaSuccess) {
        rad_mlp_destroy(m);
        return RAD_E_NOMEM;
    }
    // He-uniform initialisation from a 64-bit LCG (deterministic per seed), zero biases
    std::vector<float> h(n, 0.f);
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    for (int l = 0; l < kLayers; l++) {
        const float lim = std::sqrt(6.0f / (float)kDims[l]);
        for (size_t e = 0; e < (size_t)kDims[l + 1] * kDims[l]; e++) {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const float u = (float)((st >> 40) & 0xFFFFFF) / 16777216.0f;
            h[m->off.w[l] + e] = (2.f * u - 1.f) * lim;
        }
    }
    cudaMemcpy(m->p, h.data(), 4 * n, cudaMemcpyHostToDevice);
    cudaMemset(m->m, 0, 4 * n);
    cudaMemset(m->v, 0, 4 * n);
    for (int l = 0; l < kLayers; l++)
        if (cudaMalloc(&m->w16[l], 2 * (size_t)kNRout[l] * kKin[l]) != cudaSuccess ||
            cudaMalloc(&m->wt16[l], 2 * (size_t)kNRin[l] * kKout[l]) != cudaSuccess) {
            rad_mlp_destroy(m);
            return RAD_E_NOMEM;
        }
    k_to_bf16<<<64, 256, 0, m->stream>>>(m->p, (uint32_t)n, m->p16);
    tc_refresh(m);
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) {
        rad_mlp_destroy(m);
        return RAD_E_CUDA;
    }
    *out = m;
    return RAD_OK;
}

int rad_mlp_destroy(rad_mlp* m) {
    if (!m) return RAD_E_INVALID;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->p);
    cudaFree(m->p16);
    cudaFree(m->g);
    cudaFree(m->m);
    cudaFree(m->v);
    cudaFree(m->loss);
    cudaFree(m->tgt);
    tc_free_acts(m);
    for (int l = 0; l < kLayers; l++) {
        cudaFree(m->w16[l]);
        cudaFree(m->wt16[l]);
    }
    cudaFree(m->ctr);
    for (int l = 0; l <= kLayers; l++) {
        cudaFree(m->act[l]);
        cudaFree(m->dact[l]);
    }
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return RAD_OK;
}

uint32_t rad_mlp_param_count(void) { return (uint32_t)offsets().total; }

int rad_mlp_set_tensor_cores(rad_mlp* m, int on) {
    if (!m) return RAD_E_INVALID;
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) return RAD_E_CUDA;
    m->tc = on != 0;
    return RAD_OK;
}

int rad_mlp_get_params(rad_mlp* m, float* out) {
    if (!m || !out) return RAD_E_INVALID;
    cudaStreamSynchronize(m->stream);
    return cudaMemcpy(out, m->p, 4 * m->off.total, cudaMemcpyDeviceToHost) == cudaSuccess ? RAD_OK : RAD_E_CUDA;
}

int rad_mlp_set_params(rad_mlp* m, const float* in) {
    if (!m || !in) return RAD_E_INVALID;
    cudaStreamSynchronize(m->stream);
    if (cudaMemcpy(m->p, in, 4 * m->off.total, cudaMemcpyHostToDevice) != cudaSuccess) return RAD_E_CUDA;
    k_to_bf16<<<64, 256, 0, m->stream>>>(m->p, (uint32_t)m->off.total, m->p16);
    tc_refresh(m);
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? RAD_OK : RAD_E_CUDA;
}

int rad_mlp_predict(rad_mlp* m, const float* X, uint32_t P, float* Y) {
    if (!m || !X || !Y || P == 0) return RAD_E_INVALID;
    int rc = mlp_ensure(m, P);
    if (!rc && m->tc) rc = tc_ensure(m, P);
    if (rc) return rc;
    cudaMemcpyAsync(m->act[0], X, sizeof(float) * (size_t)P * kIn, cudaMemcpyHostToDevice, m->stream);
    const float* out = m->act[kLayers];
    if (m->tc) {
        tc_stage(m, m->act[0], P);
        if ((rc = tc_forward(m, P))) return rc;
        out = m->y;
    } else {
        mlp_forward(m, P);
    }
    cudaMemcpyAsync(Y, out, sizeof(float) * (size_t)P * kOut, cudaMemcpyDeviceToHost, m->stream);
    return (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(m->stream) == cudaSuccess) ? RAD_OK : RAD_E_CUDA;
}

int rad_mlp_gradients(rad_mlp* m, const float* X, const float* T, uint32_t P, float* grads, double* loss) {
    if (!m || !X || !T || P == 0) return RAD_E_INVALID;
    int rc = mlp_ensure(m, P);
    if (rc) return rc;
    cudaMemcpyAsync(m->act[0], X, sizeof(float) * (size_t)P * kIn, cudaMemcpyHostToDevice, m->stream);
    cudaMemcpyAsync(m->tgt, T, sizeof(float) * (size_t)P * kOut, cudaMemcpyHostToDevice, m->stream);
    if (m->tc) {
        if ((rc = tc_ensure(m, P))) return rc;
        cudaMemsetAsync(m->g, 0, sizeof(float) * m->off.total, m->stream);
        tc_stage(m, m->act[0], P);
        if ((rc = tc_forward(m, P)) || (rc = tc_backward(m, P))) return rc;
    } else {
        mlp_forward(m, P);
        mlp_backward(m, P);
    }
    double l = 0;
    if (grads) cudaMemcpyAsync(grads, m->g, 4 * m->off.total, cudaMemcpyDeviceToHost, m->stream);
    cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(m->stream) != cudaSuccess) return RAD_E_CUDA;
    if (loss) *loss = l / ((double)P * kOut);
    return RAD_OK;
}

int rad_mlp_train(rad_mlp* m, const float* X, const float* T, uint32_t P, uint32_t epochs, uint32_t batch, float lr,
                  double* final_loss, double* device_ms) {
    if (!m || !X || !T || P == 0 || batch == 0) return RAD_E_INVALID;
    // the whole data set lives on the device; batches are consecutive slices of it
    float *dX = nullptr, *dT = nullptr;
    if (cudaMalloc(&dX, sizeof(float) * (size_t)P * kIn) != cudaSuccess ||
        cudaMalloc(&dT, sizeof(float) * (size_t)P * kOut) != cudaSuccess) {
        cudaFree(dX);
        return RAD_E_NOMEM;
    }
    int rc = mlp_ensure(m, batch);
    if (!rc && m->tc) rc = tc_ensure(m, batch);
    if (rc) {
        cudaFree(dX);
        cudaFree(dT);
        return rc;
    }
    cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)P * kIn, cudaMemcpyHostToDevice, m->stream);
    cudaMemcpyAsync(dT, T, sizeof(float) * (size_t)P * kOut, cudaMemcpyHostToDevice, m->stream);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, m->stream);
    double l = 0;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    if (m->tc && rc == RAD_OK) {
        // the tensor-core engine: one captured graph per full batch (staging from the device
        // data set by the batch counter, forward, backward, Adam, BF16 weight copies, counters),
        // replayed P / batch times per epoch; a last partial batch runs the same kernels directly
        const uint32_t full = P / batch, rem = P % batch;
        const uint32_t h_ctr[2] = {m->step, 0u};
        cudaMemcpyAsync(m->ctr, h_ctr, 8, cudaMemcpyHostToDevice, m->stream);
        cudaStreamSynchronize(m->stream);
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        if (full > 0) {
            const uint32_t K = (batch + 63u) & ~63u;
            bool ok = cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                if (K > batch)
                    for (int k = 0; k < kLayers; k++)
                        cudaMemset2DAsync(m->ac[k] + batch, 2 * (size_t)K, 0, 2 * (size_t)(K - batch), kNRin[k],
                                          m->stream);
                k_tc_batch<<<(batch + 127) / 128, 128, 0, m->stream>>>(dX, dT, batch, K, m->ctr, m->ar[0],
                                                                       m->ac[0], m->tgt);
                if (tc_forward(m, batch) || tc_backward(m, batch)) ok = false;
                k_step_begin<<<1, 1, 0, m->stream>>>(m->ctr);
                k_adam_dev<<<64, 256, 0, m->stream>>>(m->p, m->g, m->m, m->v, (uint32_t)m->off.total, lr, b1, b2,
                                                      eps, m->ctr, m->p16);
                tc_refresh(m);
                k_step_end<<<1, 1, 0, m->stream>>>(m->ctr, full);
            }
            const bool ended = cudaStreamEndCapture(m->stream, &graph) == cudaSuccess;
            if (!ok || !ended || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) rc = RAD_E_CUDA;
        }
        for (uint32_t ep = 0; ep < epochs && rc == RAD_OK; ep++) {
            for (uint32_t s = 0; s < full && rc == RAD_OK; s++)
                if (cudaGraphLaunch(exec, m->stream) != cudaSuccess) rc = RAD_E_CUDA;
            if (rem && rc == RAD_OK) {
                const size_t at = (size_t)full * batch;
                cudaMemcpyAsync(m->tgt, dT + at * kOut, sizeof(float) * (size_t)rem * kOut, cudaMemcpyDeviceToDevice,
                                m->stream);
                tc_stage(m, dX + at * kIn, rem);
                if ((rc = tc_forward(m, rem)) || (rc = tc_backward(m, rem))) break;
                k_step_begin<<<1, 1, 0, m->stream>>>(m->ctr);
                k_adam_dev<<<64, 256, 0, m->stream>>>(m->p, m->g, m->m, m->v, (uint32_t)m->off.total, lr, b1, b2,
                                                      eps, m->ctr, m->p16);
                tc_refresh(m);
            }
        }
        m->step += epochs * (full + (rem ? 1u : 0u));
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
    for (uint32_t ep = 0; ep < epochs && rc == RAD_OK && !m->tc; ep++) {
        for (uint32_t at = 0; at < P; at += batch) {
            const uint32_t nb = P - at < batch ? P - at : batch;
            cudaMemcpyAsync(m->act[0], dX + (size_t)at * kIn, sizeof(float) * (size_t)nb * kIn,
                            cudaMemcpyDeviceToDevice, m->stream);
            cudaMemcpyAsync(m->tgt, dT + (size_t)at * kOut, sizeof(float) * (size_t)nb * kOut,
                            cudaMemcpyDeviceToDevice, m->stream);
            mlp_forward(m, nb);
            mlp_backward(m, nb);
            m->step++;
            const float bc1 = 1.f - std::pow(b1, (float)m->step), bc2 = 1.f - std::pow(b2, (float)m->step);
            k_adam<<<64, 256, 0, m->stream>>>(m->p, m->g, m->m, m->v, (uint32_t)m->off.total, lr, b1, b2, eps, bc1,
                                              bc2, m->p16);
        }
    }
    cudaEventRecord(e1, m->stream);
    cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream);
    const bool ok = rc == RAD_OK && cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(m->stream) == cudaSuccess;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(dX);
    cudaFree(dT);
    if (!ok) return RAD_E_CUDA;
    if (final_loss) *final_loss = l / ((double)(P - (P - 1) / batch * batch) * kOut);
    if (device_ms) *device_ms = ms;
    return RAD_OK;
}

}  // extern "C"
