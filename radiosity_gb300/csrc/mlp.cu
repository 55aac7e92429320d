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

#include <cmath>
#include <cstring>
#include <vector>

#include "radiosity.h"
#include "rad_internal.cuh"

namespace {

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
};

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
    if (cudaSetDevice(device) != cudaSuccess) return RAD_E_CUDA;
    rad_mlp* m = new rad_mlp();
    m->device = device;
    m->off = offsets();
    const size_t n = m->off.total;
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&m->p, 4 * n) != cudaSuccess || cudaMalloc(&m->p16, 2 * n) != cudaSuccess ||
        cudaMalloc(&m->g, 4 * n) != cudaSuccess || cudaMalloc(&m->m, 4 * n) != cudaSuccess ||
        cudaMalloc(&m->v, 4 * n) != cudaSuccess || cudaMalloc(&m->loss, 8) != cudaSuccess) {
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
    k_to_bf16<<<64, 256, 0, m->stream>>>(m->p, (uint32_t)n, m->p16);
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
    for (int l = 0; l <= kLayers; l++) {
        cudaFree(m->act[l]);
        cudaFree(m->dact[l]);
    }
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return RAD_OK;
}

uint32_t rad_mlp_param_count(void) { return (uint32_t)offsets().total; }

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
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? RAD_OK : RAD_E_CUDA;
}

int rad_mlp_predict(rad_mlp* m, const float* X, uint32_t P, float* Y) {
    if (!m || !X || !Y || P == 0) return RAD_E_INVALID;
    int rc = mlp_ensure(m, P);
    if (rc) return rc;
    cudaMemcpyAsync(m->act[0], X, sizeof(float) * (size_t)P * kIn, cudaMemcpyHostToDevice, m->stream);
    mlp_forward(m, P);
    cudaMemcpyAsync(Y, m->act[kLayers], sizeof(float) * (size_t)P * kOut, cudaMemcpyDeviceToHost, m->stream);
    return (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(m->stream) == cudaSuccess) ? RAD_OK : RAD_E_CUDA;
}

int rad_mlp_gradients(rad_mlp* m, const float* X, const float* T, uint32_t P, float* grads, double* loss) {
    if (!m || !X || !T || P == 0) return RAD_E_INVALID;
    int rc = mlp_ensure(m, P);
    if (rc) return rc;
    cudaMemcpyAsync(m->act[0], X, sizeof(float) * (size_t)P * kIn, cudaMemcpyHostToDevice, m->stream);
    cudaMemcpyAsync(m->tgt, T, sizeof(float) * (size_t)P * kOut, cudaMemcpyHostToDevice, m->stream);
    mlp_forward(m, P);
    mlp_backward(m, P);
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
    for (uint32_t ep = 0; ep < epochs; ep++) {
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
    const bool ok = cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(m->stream) == cudaSuccess;
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
