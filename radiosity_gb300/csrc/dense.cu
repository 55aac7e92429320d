// Dense form-factor capture and the gathering solve B = E + rho o (F B).
//
// F rows come from the hemicube pipeline (exact sums, one row per shooter).  They
// are kept as FP32 rows and as BF16 rows with one FP32 scale per row
// (F_ij ~= scale_i * bf16_ij, scale_i = max_j F_ij).  The solve is mixed-precision
// iterative refinement:
//     r  = E + rho o (F32 B) - B                     FP32 GEMM (k_sgemm_resid), FP64 norms
//     d <- r + rho o (scale o (F16 d))   (m sweeps)  BF16 tcgen05 GEMM (k_gemm_tc)
//     B <- B + d
// Right-hand sides are column-major: column c of an N x R block is contiguous, and
// column c uses the reflectance channel c % 3.
//
// k_gemm_tc is a warp-specialised tcgen05 GEMM for C[128 x NR] tiles (two of them per CTA,
// sharing each NR x 64 tile of B, for the solve's sweeps with NR >= 128): warp 0 issues
// TMA loads (128B swizzle) of 128 x 64 tiles of F16 and an NR x 64 tile of the
// transposed operand into a 4-stage ring, warp 1 issues tcgen05.mma (BF16 x BF16 ->
// FP32 in TMEM) and frees stages with tcgen05.commit, warp 2 owns the TMEM
// allocation, and warps 4-7 read the accumulator with tcgen05.ld and run the fused
// epilogue.  When the row tiles alone would leave SMs idle (80 two-tile CTAs on 152 SMs at
// N = 20k), K is split (a tile's splits are neighbours in launch order); each split writes
// its FP32 partial sums and k_tc_finalize adds them in split order (deterministic) before the
// same epilogue.  The streamed matrix is loaded with an L2 evict-first policy.  Every
// mbarrier wait is bounded by wall-clock time; a timeout sets the error word and the kernel
// drains and frees its TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>
#include <stdint.h>

#include <cmath>

#include "rad_internal.cuh"
#include "pipe.cuh"

namespace rad {

// ---------------------------------------------------------------------------
// Row capture: exact sums -> FP32 rows, BF16 rows + per-row scale
// ---------------------------------------------------------------------------
// One CTA per captured row: exact sums -> FP32 row (optional), BF16 row scaled by the
// row maximum, and the scale.  The sums are zeroed after their last read, ready for the
// next chunk of rows.
__global__ void __launch_bounds__(256) k_dense_rows(unsigned long long* __restrict__ Fq, uint32_t n, uint32_t ld,
                                                    uint32_t first, float* F32, __nv_bfloat16* F16, float* scale) {
    const uint32_t r = blockIdx.x;  // row within the batch
    unsigned long long* src = Fq + (size_t)r * n;
    const size_t row = (size_t)(first + r);
    __shared__ float red[256];
    float mx = 0.f;
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
        const float f = __ull2float_rn(src[j]) * 0x1p-61f;
        if (F32) F32[row * ld + j] = f;
        mx = fmaxf(mx, f);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (uint32_t o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    const float s = red[0] > 0.f ? red[0] : 1.0f;
    const float inv = 1.0f / s;
    for (uint32_t j = threadIdx.x; j < ld; j += blockDim.x) {
        float f = 0.f;
        if (j < n) {
            f = __ull2float_rn(src[j]) * 0x1p-61f;
            src[j] = 0ull;
        }
        F16[row * ld + j] = __float2bfloat16_rn(f * inv);
    }
    if (threadIdx.x == 0) scale[row] = s;
}

void launch_dense_rows(unsigned long long* Fq, uint32_t count, uint32_t n, uint32_t ld, uint32_t first,
                       float* F32, __nv_bfloat16* F16, float* scale, cudaStream_t s) {
    k_dense_rows<<<count, 256, 0, s>>>(Fq, n, ld, first, F32, F16, scale);
}

// ---------------------------------------------------------------------------
// FP32 residual GEMM: r[c][i] = E[c][i] + rho_i[c%3] * sum_j F[i][j] X[c][j] - X[c][i]
// (with weights w and inv_a: the sum is over F[i][j] w_j X[c][j] and is multiplied by inv_a_i;
// the shoot form passes the transposed rows, w = A and inv_a = 1 / A)
// 128 (rows) x 64 (columns) tiles, 128 threads with 8 x 8 outputs each (four FMAs per
// shared-memory word loaded), 16-deep k slabs double-buffered in shared memory, the next
// slab's global loads in flight during the current slab's FMAs, one barrier per slab.
// Compensated sum: every 64 k the thread's FP32 chunk sums are added to their high parts (one
// word per output, in shared memory) with Knuth's TwoSum, and the rounding error of that add
// starts the next chunk, so the sum over N ~ 20k terms carries the rounding of 64-term
// partials instead of growing like sqrt(N) * eps: the refinement's FP32 residual then agrees
// with an FP64 evaluation to well below the 1e-6 tolerance.  Column norms: nrm[c] += r^2
// (FP64 atomics).  Entries of F at columns >= n (the row padding up to ld) are never read.
// ---------------------------------------------------------------------------
constexpr int kRBM = 128, kRBN = 64, kRBK = 16, kRComp = 4, kRThreads = 128;
constexpr int kRAs = kRBK * (kRBM + 4), kRBs = kRBK * (kRBN + 4);   // one buffer, floats
constexpr int kRSmem = (2 * kRAs + 2 * kRBs + kRBM * kRBN) * 4;     // 58,368 B

__global__ void __launch_bounds__(kRThreads, 3) k_sgemm_resid(const float* __restrict__ F, uint32_t n, uint32_t ld,
                                                              const float* __restrict__ X,
                                                              const float* __restrict__ E,
                                                              const float4* __restrict__ rho, uint32_t R, float* r,
                                                              double* nrm, const float* __restrict__ w,
                                                              const float* __restrict__ inv_a, uint32_t nsplit,
                                                              float* __restrict__ part) {
    extern __shared__ __align__(16) float s_rs[];
    float* As = s_rs;                    // [2][kRBK][kRBM + 4], As[k][i]
    float* Bs = As + 2 * kRAs;           // [2][kRBK][kRBN + 4], Bs[k][c]
    float* Hs = Bs + 2 * kRBs;           // [64 outputs][128 threads]: high parts
    const uint32_t i0 = blockIdx.x * kRBM, c0 = blockIdx.y * kRBN;
    const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;  // columns tx*8.., rows ty*8..
    // global -> register staging of one slab: A rows (tid >> 2) + 32 q, k (tid & 3) * 4 .. + 3;
    // B columns (tid >> 2) + 32 q, the same k
    const int lr = tid >> 2, lk = (tid & 3) * 4;
    float4 ra[4], rb[2];
    auto load = [&](uint32_t k0) {
        const uint32_t k = k0 + (uint32_t)lk;
        float4 wv = make_float4(1.f, 1.f, 1.f, 1.f);
        if (w) {
            wv.x = k < n ? w[k] : 0.f;
            wv.y = k + 1 < n ? w[k + 1] : 0.f;
            wv.z = k + 2 < n ? w[k + 2] : 0.f;
            wv.w = k + 3 < n ? w[k + 3] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t i = i0 + (uint32_t)(lr + 32 * q);
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (i < n) {
                const float* src = F + (size_t)i * ld + k;
                if (k + 3 < n) v = *reinterpret_cast<const float4*>(src);  // ld % 4 == 0, k % 4 == 0
                else {
                    if (k < n) v.x = src[0];
                    if (k + 1 < n) v.y = src[1];
                    if (k + 2 < n) v.z = src[2];
                }
            }
            ra[q] = v;
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const uint32_t c = c0 + (uint32_t)(lr + 32 * q);
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (c < R) {
                const float* src = X + (size_t)c * n + k;  // column c of X: n floats, no alignment
                if (k < n) v.x = src[0] * wv.x;
                if (k + 1 < n) v.y = src[1] * wv.y;
                if (k + 2 < n) v.z = src[2] * wv.z;
                if (k + 3 < n) v.w = src[3] * wv.w;
            }
            rb[q] = v;
        }
    };
    auto store = [&](int buf) {
        float* A = As + buf * kRAs;
        float* B = Bs + buf * kRBs;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int i = lr + 32 * q;
            A[(lk + 0) * (kRBM + 4) + i] = ra[q].x;
            A[(lk + 1) * (kRBM + 4) + i] = ra[q].y;
            A[(lk + 2) * (kRBM + 4) + i] = ra[q].z;
            A[(lk + 3) * (kRBM + 4) + i] = ra[q].w;
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int c = lr + 32 * q;
            B[(lk + 0) * (kRBN + 4) + c] = rb[q].x;
            B[(lk + 1) * (kRBN + 4) + c] = rb[q].y;
            B[(lk + 2) * (kRBN + 4) + c] = rb[q].z;
            B[(lk + 3) * (kRBN + 4) + c] = rb[q].w;
        }
    };
    float acc[8][8];
#pragma unroll
    for (int p = 0; p < 8; p++)
#pragma unroll
        for (int q = 0; q < 8; q++) {
            acc[p][q] = 0.f;
            Hs[(p * 8 + q) * kRThreads + tid] = 0.f;
        }
    // split-K: blockIdx.z takes slabs [sl0, sl1)
    const uint32_t nslabs = (n + kRBK - 1) / kRBK;
    const uint32_t sl0 = blockIdx.z * nslabs / nsplit, sl1 = (blockIdx.z + 1) * nslabs / nsplit;
    load(sl0 * kRBK);
    store(0);
    __syncthreads();
    for (uint32_t sl = sl0; sl < sl1; sl++) {
        const int cur = (int)((sl - sl0) & 1u);
        const bool more = sl + 1 < sl1;
        if (more) load((sl + 1) * kRBK);  // in flight during the FMAs below
        const float* A = As + cur * kRAs + ty * 8;
        const float* B = Bs + cur * kRBs + tx * 8;
#pragma unroll
        for (int kk = 0; kk < kRBK; kk++) {
            const float4 a0 = *reinterpret_cast<const float4*>(A + kk * (kRBM + 4));
            const float4 a1 = *reinterpret_cast<const float4*>(A + kk * (kRBM + 4) + 4);
            const float4 b0 = *reinterpret_cast<const float4*>(B + kk * (kRBN + 4));
            const float4 b1 = *reinterpret_cast<const float4*>(B + kk * (kRBN + 4) + 4);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int p = 0; p < 8; p++)
#pragma unroll
                for (int q = 0; q < 8; q++) acc[p][q] = fmaf(a[p], bb[q], acc[p][q]);
        }
        if (more) store(cur ^ 1);  // the other buffer: last read before the previous barrier
        if ((sl + 1 - sl0) % kRComp == 0 || !more) {
#pragma unroll
            for (int p = 0; p < 8; p++)
#pragma unroll
                for (int q = 0; q < 8; q++) {  // TwoSum(hi, acc): the error starts the next chunk
                    float* hp = Hs + (p * 8 + q) * kRThreads + tid;
                    const float h = *hp, b = acc[p][q];
                    const float s = h + b, bv = s - h;
                    acc[p][q] = (h - (s - bv)) + (b - bv);
                    *hp = s;
                }
        }
        __syncthreads();
    }
    if (nsplit > 1) {  // the split's compensated sums (hi, lo) for k_sgemm_resid_finalize
        float* phi = part + (size_t)blockIdx.z * R * n;
        float* plo = part + (size_t)(nsplit + blockIdx.z) * R * n;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const uint32_t c = c0 + (uint32_t)(tx * 8 + q);
            if (c >= R) continue;
#pragma unroll
            for (int p = 0; p < 8; p++) {
                const uint32_t i = i0 + (uint32_t)(ty * 8 + p);
                if (i >= n) continue;
                phi[(size_t)c * n + i] = Hs[(p * 8 + q) * kRThreads + tid];
                plo[(size_t)c * n + i] = acc[p][q];
            }
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const uint32_t c = c0 + (uint32_t)(tx * 8 + q);
        double part = 0;
        if (c < R) {
            const int ch = (int)(c % 3);
#pragma unroll
            for (int p = 0; p < 8; p++) {
                const uint32_t i = i0 + (uint32_t)(ty * 8 + p);
                if (i >= n) continue;
                const float4 rh = rho[i];
                const float rr = ch == 0 ? rh.x : (ch == 1 ? rh.y : rh.z);
                const float sum = (Hs[(p * 8 + q) * kRThreads + tid] + acc[p][q]) * (inv_a ? inv_a[i] : 1.0f);
                const float v = E[(size_t)c * n + i] + rr * sum - X[(size_t)c * n + i];
                r[(size_t)c * n + i] = v;
                part += (double)v * (double)v;
            }
        }
        // lanes with the same tx (lane ^ 8, lane ^ 16) hold the same columns
        part += __shfl_xor_sync(0xffffffffu, part, 8);
        part += __shfl_xor_sync(0xffffffffu, part, 16);
        if (nrm && c < R && (threadIdx.x & 31) < 8) atomicAdd(&nrm[c], part);
    }
}

// Self-test of the bounded pipeline wait: one thread waits on an mbarrier that nothing
// arrives on.  The wait gives up after limit_ns and sets *err, which is the path every
// pipeline wait takes when its copies never land; the kernel then returns normally.
__global__ void k_wait_selftest(uint32_t* err, unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_wait(&bar, 0, err, limit_ns);
    }
}

int launch_wait_selftest(uint32_t* err, unsigned long long limit_ns, cudaStream_t s) {
    k_wait_selftest<<<1, 32, 0, s>>>(err, limit_ns);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// The splits' (hi, lo) pairs added in split order with TwoSum, then the residual and the norms:
// block (x, c) takes rows x * 256 .. + 255 of column c (one FP64 atomic per block).
__global__ void __launch_bounds__(256) k_sgemm_resid_finalize(const float* __restrict__ part, uint32_t nsplit,
                                                              uint32_t n, const float* __restrict__ X,
                                                              const float* __restrict__ E,
                                                              const float4* __restrict__ rho, uint32_t R, float* r,
                                                              double* nrm, const float* __restrict__ inv_a) {
    const uint32_t c = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ double s_part[8];
    double sq = 0.0;
    if (i < n) {
        const size_t at = (size_t)c * n + i, stride = (size_t)R * n;
        float H = 0.f, L = 0.f;
        for (uint32_t sp = 0; sp < nsplit; sp++) {
            const float h = part[sp * stride + at], l = part[(nsplit + sp) * stride + at];
            const float s2 = H + h, bv = s2 - H;
            L += ((H - (s2 - bv)) + (h - bv)) + l;
            H = s2;
        }
        const float4 rh = rho[i];
        const int ch = (int)(c % 3);
        const float rr = ch == 0 ? rh.x : (ch == 1 ? rh.y : rh.z);
        const float sum = (H + L) * (inv_a ? inv_a[i] : 1.0f);
        const float v = E[at] + rr * sum - X[at];
        r[at] = v;
        sq = (double)v * (double)v;
    }
    if (!nrm) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < 8; k++) t += s_part[k];
        atomicAdd(&nrm[c], t);
    }
}

// K splits of the tiled residual (R > 4): the count (1..16, at least 32 slabs each) that
// balances the waves of 3 CTAs per SM against the partial sums written and read back.
static uint32_t sgemm_resid_splits(uint32_t n, uint32_t R) {
    const uint32_t ctas = ((n + kRBM - 1) / kRBM) * ((R + kRBN - 1) / kRBN), nslabs = (n + kRBK - 1) / kRBK;
    const double slots = 152.0 * 3.0;
    uint32_t best = 1;
    double best_cost = 1e300;
    for (uint32_t sp = 1; sp <= 16; sp++) {
        if (sp > 1 && nslabs / sp < 32) break;
        const double work = (double)ctas * sp;
        const double fill = work / (std::ceil(work / slots) * slots);
        const double cost = 1.0 / fill + 60.0 * sp / (double)n;
        if (cost < best_cost - 1e-12) {
            best_cost = cost;
            best = sp;
        }
    }
    return best;
}

size_t sgemm_resid_scratch_floats(uint32_t R, uint32_t ld) {
    if (R <= kResidStreamRhs) return (size_t)kResidStreamRhs * ld;
    const uint32_t sp = sgemm_resid_splits(ld, R);  // sized by ld >= n, as the launch plans it
    return sp > 1 ? (size_t)2 * sp * R * ld : 0;
}

void launch_sgemm_resid(const float* F, uint32_t n, uint32_t ld, const float* X, const float* E, const float4* rho,
                        uint32_t R, float* r, double* nrm, float* scratch, uint32_t* err, cudaStream_t s,
                        const float* w, const float* inv_a) {
    if (R <= kResidStreamRhs) {
        launch_resid_stream(F, n, ld, X, E, rho, R, r, nrm, scratch, err, s, w, inv_a);
        return;
    }
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_sgemm_resid, cudaFuncAttributeMaxDynamicSharedMemorySize, kRSmem);
    (void)attr;  // a failure shows as the launch error
    // the splits the scratch was sized for (sgemm_resid_scratch_floats); null scratch: one split
    const uint32_t sp = scratch ? sgemm_resid_splits(ld, R) : 1u;
    dim3 grid((n + kRBM - 1) / kRBM, (R + kRBN - 1) / kRBN, sp);
    k_sgemm_resid<<<grid, kRThreads, kRSmem, s>>>(F, n, ld, X, E, rho, R, r, nrm, w, inv_a, sp, scratch);
    if (sp > 1)
        k_sgemm_resid_finalize<<<dim3((n + 255) / 256, R), 256, 0, s>>>(scratch, sp, n, X, E, rho, R, r, nrm, inv_a);
}

// ---------------------------------------------------------------------------
// Shooting-form residual: the progressive shooter distributes patch i's power with
// F_ji = F_ij A_i / A_j (source/Main.cpp:1268-1276 with the area ratio), so its fixed
// point solves B_j = E_j + rho_j (sum_i F_ij A_i B_i) / A_j.  k_colsum_area forms
// acc[c][j] += sum_i F_ij A_i X[c][i] over a slab of 1024 rows per CTA row (FP32 in
// the slab, FP64 atomics across slabs); k_shoot_resid finishes r.
// ---------------------------------------------------------------------------
constexpr uint32_t kColSlab = 1024;
constexpr uint32_t kColRhs = 4;

__global__ void __launch_bounds__(256) k_colsum_area(const float* __restrict__ F, uint32_t n, uint32_t ld,
                                                     const float* __restrict__ X, const float* __restrict__ area,
                                                     uint32_t R, uint32_t c0, double* acc) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i0 = blockIdx.y * kColSlab, i1 = min(n, i0 + kColSlab);
    const uint32_t nc = min(kColRhs, R - c0);
    __shared__ float y[kColRhs][64];
    float s[kColRhs] = {0.f, 0.f, 0.f, 0.f};
    for (uint32_t b0 = i0; b0 < i1; b0 += 64) {
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < kColRhs * 64; e += blockDim.x) {
            const uint32_t c = e / 64, i = b0 + e % 64;
            y[c][e % 64] = (c < nc && i < i1) ? area[i] * X[(size_t)(c0 + c) * n + i] : 0.f;
        }
        __syncthreads();
        if (j < n) {
            const uint32_t m = min(64u, i1 - b0);
            for (uint32_t q = 0; q < m; q++) {
                const float f = F[(size_t)(b0 + q) * ld + j];
#pragma unroll
                for (uint32_t c = 0; c < kColRhs; c++) s[c] = fmaf(f, y[c][q], s[c]);
            }
        }
    }
    if (j < n)
        for (uint32_t c = 0; c < nc; c++) atomicAdd(&acc[(size_t)(c0 + c) * n + j], (double)s[c]);
}

__global__ void k_shoot_resid(const double* __restrict__ acc, const float* __restrict__ X, const float* __restrict__ E,
                              const float4* __restrict__ rho, const float* __restrict__ area, uint32_t n, uint32_t R,
                              float* r) {
    const size_t total = (size_t)n * R;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(e / n), j = (uint32_t)(e % n);
        const float4 rh = rho[j];
        const int ch = (int)(c % 3);
        const double rr = ch == 0 ? rh.x : (ch == 1 ? rh.y : rh.z);
        const double a = area[j];
        const double v = (double)E[e] + (a > 0 ? rr * acc[e] / a : 0.0) - (double)X[e];
        r[e] = (float)v;
    }
}

void launch_shoot_resid(const float* F, uint32_t n, uint32_t ld, const float* X, const float* E, const float4* rho,
                        const float* area, uint32_t R, double* acc, float* r, cudaStream_t s) {
    cudaMemsetAsync(acc, 0, sizeof(double) * (size_t)n * R, s);
    dim3 grid((n + 255) / 256, (n + kColSlab - 1) / kColSlab);
    for (uint32_t c0 = 0; c0 < R; c0 += kColRhs) k_colsum_area<<<grid, 256, 0, s>>>(F, n, ld, X, area, R, c0, acc);
    k_shoot_resid<<<152 * 4, 256, 0, s>>>(acc, X, E, rho, area, n, R, r);
}

// BF16 transposed copy of a column-major N x R block: Xt[c][j] (ld columns, zero padded),
// each value multiplied by w[j] when weights are given.
__global__ void k_pack_bf16(const float* __restrict__ X, uint32_t n, uint32_t R, uint32_t ld, __nv_bfloat16* Xt,
                            uint32_t Rpad, const float* __restrict__ w) {
    const size_t total = (size_t)Rpad * ld;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(e / ld), j = (uint32_t)(e % ld);
        Xt[e] = __float2bfloat16_rn((c < R && j < n) ? X[(size_t)c * n + j] * (w ? w[j] : 1.0f) : 0.f);
    }
}

void launch_pack_bf16(const float* X, uint32_t n, uint32_t R, uint32_t ld, __nv_bfloat16* Xt, uint32_t Rpad,
                      cudaStream_t s, const float* w) {
    k_pack_bf16<<<152 * 8, 256, 0, s>>>(X, n, R, ld, Xt, Rpad, w);
}

// ---------------------------------------------------------------------------
// Shoot-form operands: dst[i][j] = src[j][i] for i, j < n (square n x n blocks of pitch ld),
// zeros in dst's padding columns [n, ld).  32 x 32 tiles through shared memory: both the
// reads and the writes are row segments.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_transpose(const T* __restrict__ src, uint32_t n, uint32_t ld, T* dst) {
    __shared__ T tile[32][33];
    const uint32_t j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;  // dst columns j0.., rows i0..
    const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (uint32_t y = ty; y < 32; y += 8) {  // src row j0 + y, columns i0 + tx
        const uint32_t j = j0 + y, i = i0 + tx;
        tile[y][tx] = (j < n && i < n) ? src[(size_t)j * ld + i] : T(0.0f);
    }
    __syncthreads();
    for (uint32_t y = ty; y < 32; y += 8) {
        const uint32_t i = i0 + y, j = j0 + tx;
        if (i < n && j < ld) dst[(size_t)i * ld + j] = tile[tx][y];
    }
}

// inv_a_i = 1 / A_i (0 for a degenerate patch), w_i = s_i A_i (the BF16 rows' scale times the area).
__global__ void k_shoot_weights(const float* __restrict__ area, const float* __restrict__ scale, uint32_t n,
                                float* __restrict__ inv_a, float* __restrict__ w) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float a = area[i];
        inv_a[i] = a > 0.f ? 1.0f / a : 0.f;
        w[i] = scale[i] * a;
    }
}

void launch_shoot_form(uint32_t n, uint32_t ld, const float* F32, float* F32T, const __nv_bfloat16* F16,
                       __nv_bfloat16* F16T, const float* area, const float* scale, float* inv_a, float* w,
                       cudaStream_t s) {
    const dim3 grid(ld / 32 + (ld % 32 != 0), (n + 31) / 32);
    if (F32 && F32T) k_transpose<float><<<grid, 256, 0, s>>>(F32, n, ld, F32T);
    k_transpose<__nv_bfloat16><<<grid, 256, 0, s>>>(F16, n, ld, F16T);
    k_shoot_weights<<<(n + 255) / 256, 256, 0, s>>>(area, scale, n, inv_a, w);
}

__global__ void k_axpy(float* __restrict__ y, const float* __restrict__ x, size_t total) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        y[e] = y[e] + x[e];
}

void launch_axpy(float* y, const float* x, size_t total, cudaStream_t s) { k_axpy<<<152 * 8, 256, 0, s>>>(y, x, total); }

// ---------------------------------------------------------------------------
// tcgen05 BF16 GEMM
// ---------------------------------------------------------------------------
constexpr int kTcM = 128, kTcBK = 64, kTcStages = 4;
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// The same load with an L2 cache policy (the streamed matrix is marked evict-first, so that it
// does not push the shared right-hand sides and the split-K partial sums out of L2).
__device__ __forceinline__ void tma_load_2d_hint(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar,
                                                 uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1 << 46;            // descriptor version
    d |= (uint64_t)2 << 61;            // SWIZZLE_128B
    return d;
}

// MT row tiles of 128 share each B tile (MT = 2 for wide B: half the B bytes per A byte).
template <int NR, int MT = 1>
struct TcShape {
    static constexpr uint32_t kA = kTcM * kTcBK * 2;   // one 128-row A tile
    static constexpr uint32_t kB = NR * kTcBK * 2;
    static constexpr uint32_t kStage = MT * kA + kB;
    static constexpr uint32_t kCols = NR <= 32 ? 32 : (NR <= 64 ? 64 : (NR <= 128 ? 128 : 256));
    // 1 KB header (mbarriers, TMEM slot), the stage ring, 1 KB of alignment slack; at most
    // kTcStages stages and 227 KB
    static constexpr uint32_t kMaxStages =
        (227u * 1024u - 2048u) / kStage < (uint32_t)kTcStages ? (227u * 1024u - 2048u) / kStage : (uint32_t)kTcStages;
    static constexpr uint32_t kSmem = kMaxStages * kStage + 2048;
    static constexpr uint32_t smem_for(uint32_t stages) { return stages * kStage + 2048; }
    // instruction descriptor: D f32, A/B bf16, K-major both, N = NR, M = 128
    static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NR >> 3) << 17) |
                                       ((uint32_t)(kTcM >> 4) << 24);
};

// Row tiles per CTA: two (sharing each B tile) for the solve's sweeps (modes 0, 1) with B at
// least 128 wide, else one.
__host__ __device__ constexpr uint32_t tc_mt(uint32_t NR, int mode) { return (NR >= 128 && mode <= 1) ? 2u : 1u; }

// One output element of the network modes (2-5) of TcEpilogue; y = the FP32 accumulator.
__device__ __forceinline__ void net_store(const TcEpilogue& ep, uint32_t row, uint32_t c, float y) {
    if (ep.mode == 3) {
        ep.out[(size_t)row * ep.R + c] = y + ep.bias[c];
        return;
    }
    if (ep.mode == 5) {
        ep.out[(size_t)row * ep.ldr + c] = y;
        return;
    }
    if (ep.mode == 2) y = fmaxf(y + ep.bias[c], 0.f);
    else if (!(__bfloat162float(ep.mask[(size_t)row * ep.ldm + c]) > 0.f)) y = 0.f;  // mode 4
    const __nv_bfloat16 h = __float2bfloat16_rn(y);
    ep.out16r[(size_t)row * ep.ldr + c] = h;
    ep.out16[(size_t)c * ep.ld16 + row] = h;
}

__device__ __forceinline__ void net_epilogue(const TcEpilogue& ep, uint32_t row, int c0, const uint32_t* v) {
    if ((ep.mode == 2 || ep.mode == 4) && (uint32_t)c0 + 32u <= ep.R) {
        // the row's 32 BF16 values go out as four 16-byte stores (and the mask comes in as four
        // 16-byte loads); the column-major copy is one element per lane, 32 rows per store
        uint4 mk[4];
        if (ep.mode == 4) {
            const uint4* ms = reinterpret_cast<const uint4*>(ep.mask + (size_t)row * ep.ldm + c0);
#pragma unroll
            for (int q = 0; q < 4; q++) mk[q] = ms[q];
        }
        const __nv_bfloat16* mh = reinterpret_cast<const __nv_bfloat16*>(mk);
        uint32_t packed[16];
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
            float y0 = __uint_as_float(v[j]), y1 = __uint_as_float(v[j + 1]);
            if (ep.mode == 2) {
                y0 = fmaxf(y0 + ep.bias[c0 + j], 0.f);
                y1 = fmaxf(y1 + ep.bias[c0 + j + 1], 0.f);
            } else {
                if (!(__bfloat162float(mh[j]) > 0.f)) y0 = 0.f;
                if (!(__bfloat162float(mh[j + 1]) > 0.f)) y1 = 0.f;
            }
            const __nv_bfloat162 h = __floats2bfloat162_rn(y0, y1);
            packed[j / 2] = *reinterpret_cast<const uint32_t*>(&h);
            ep.out16[(size_t)(c0 + j) * ep.ld16 + row] = h.x;
            ep.out16[(size_t)(c0 + j + 1) * ep.ld16 + row] = h.y;
        }
        uint4* dst = reinterpret_cast<uint4*>(ep.out16r + (size_t)row * ep.ldr + c0);
#pragma unroll
        for (int q = 0; q < 4; q++)
            dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
        return;
    }
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const uint32_t c = (uint32_t)(c0 + j);
        if (c >= ep.R) break;
        net_store(ep, row, c, __uint_as_float(v[j]));
    }
}

// nst: stages of the TMA ring (2..kTcStages); a short K needs fewer, and the smaller shared
// footprint lets two CTAs share an SM.
template <int NR, int MT>
__global__ void __launch_bounds__(256, 2) k_gemm_tc(const __grid_constant__ CUtensorMap tmA,
                                                    const __grid_constant__ CUtensorMap tmB, uint32_t kblocks,
                                                    uint32_t nst, TcEpilogue ep) {
    using S = TcShape<NR, MT>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* hdr = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* full = reinterpret_cast<uint64_t*>(hdr);
    uint64_t* empty = full + kTcStages;
    uint64_t* accum = empty + kTcStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
    uint8_t* smem = hdr + 1024;  // stage s at smem + s * kStage (1024-aligned for the 128B swizzle)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // split-K: block x is split x % nsplit of CTA tile x / nsplit (MT x 128 rows) and takes K
    // blocks [kb0, kb1); a tile's splits are neighbours in launch order, so they run together
    const uint32_t nsplit = (ep.partial && ep.ksplit > 1) ? ep.ksplit : 1u;
    const uint32_t split = blockIdx.x % nsplit, m0 = (blockIdx.x / nsplit) * (MT * kTcM);
    const uint32_t kb0 = split * kblocks / nsplit, kb1 = (split + 1) * kblocks / nsplit;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < nst; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(MT * S::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *tmem_slot;
    if (warp == 0 && lane == 0) {
        uint64_t stream_policy;
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(stream_policy));
        for (uint32_t kb = kb0; kb < kb1; kb++) {
            const uint32_t s = (kb - kb0) % nst, round = (kb - kb0) / nst;
            if (!mbar_wait(&empty[s], (round & 1u) ^ 1u, ep.err)) break;
            mbar_expect_tx(&full[s], S::kStage);
#pragma unroll
            for (int t = 0; t < MT; t++)
                tma_load_2d_hint(smem + s * S::kStage + t * S::kA, &tmA, (int)(kb * kTcBK), (int)(m0 + t * kTcM),
                                 &full[s], stream_policy);
            tma_load_2d(smem + s * S::kStage + MT * S::kA, &tmB, (int)(kb * kTcBK), 0, &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        bool ok = true;
        for (uint32_t kb = kb0; kb < kb1; kb++) {
            const uint32_t s = (kb - kb0) % nst, round = (kb - kb0) / nst;
            if (!mbar_wait(&full[s], round & 1u, ep.err)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t b0 = sw128_desc(smem_u32(smem + s * S::kStage + MT * S::kA));
#pragma unroll
            for (int t = 0; t < MT; t++) {
                const uint64_t a0 = sw128_desc(smem_u32(smem + s * S::kStage + t * S::kA));
#pragma unroll
                for (int k = 0; k < kTcBK / 16; k++) {
                    const uint32_t acc = ((kb - kb0) | (uint32_t)k) ? 1u : 0u;
                    asm volatile(
                        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(
                            taddr + (uint32_t)t * S::kCols),
                        "l"(a0 + (uint64_t)(2 * k)), "l"(b0 + (uint64_t)(2 * k)), "r"(S::kIdesc), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&empty[s]))
                         : "memory");
        }
        if (ok)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(accum))
                         : "memory");
    } else if (warp >= 4) {
        const int wq = warp - 4;
        if (mbar_wait(accum, 0, ep.err)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
          for (int t = 0; t < MT; t++) {
            const uint32_t row = m0 + (uint32_t)(t * kTcM + wq * 32 + lane);
            const bool live = row < ep.n;
            const float sc = (live && ep.scale) ? ep.scale[row] : 1.0f;
            const float ws = (live && ep.wscale) ? ep.wscale[row] : 1.0f;
            float4 rh = make_float4(0, 0, 0, 0);
            if (live && ep.mode == 1) rh = ep.rho[row];
#pragma unroll 1
            for (int c0 = 0; c0 < NR; c0 += 32) {
                uint32_t v[32];
                const uint32_t ta = taddr + (uint32_t)t * S::kCols + ((uint32_t)(wq * 32) << 16) + (uint32_t)c0;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(ta));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (!live) continue;
                if (nsplit == 1 && ep.mode >= 2) {
                    net_epilogue(ep, row, c0, v);
                    continue;
                }
                if (nsplit > 1) {  // raw partial sums; k_tc_finalize adds the splits in order
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const uint32_t c = (uint32_t)(c0 + j);
                        if (c >= ep.R) break;
                        ep.partial[((size_t)split * ep.R + c) * ep.n + row] = __uint_as_float(v[j]);
                    }
                    continue;
                }
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const uint32_t c = (uint32_t)(c0 + j);
                    if (c >= ep.R) break;
                    float y = sc * __uint_as_float(v[j]);
                    if (ep.mode == 1) {
                        const int ch = (int)(c % 3);
                        const float rr = ch == 0 ? rh.x : (ch == 1 ? rh.y : rh.z);
                        y = ep.resid[(size_t)c * ep.n + row] + rr * y;
                    }
                    ep.out[(size_t)c * ep.n + row] = y;
                    if (ep.out16) ep.out16[(size_t)c * ep.ld16 + row] = __float2bfloat16_rn(y * ws);
                }
            }
          }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 2) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(MT * S::kCols)
                     : "memory");
    }
}

// Host side: tensor maps through the driver entry point (no libcuda link needed).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Looked up once; function-local static initialisation is thread-safe, so contexts driven
// from several host threads share the lookup.
static EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(p);
        return EncodeTiledFn(nullptr);
    }();
    return fn;
}

// 2-D bf16 tensor map over rows x cols (row length ld elements, ld % 64 == 0), box box_rows x 64.
static bool make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t ld, uint32_t box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || (ld % 64) != 0 || (reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
    const cuuint64_t dims[2] = {ld, rows};
    const cuuint64_t strides[1] = {ld * 2};
    const cuuint32_t box[2] = {64, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Split-K epilogue: y = scale * (sum of the splits' partial sums, in split order), then the
// same update and BF16 copy as the fused epilogue.  Element (c, row) per thread.
__global__ void k_tc_finalize(TcEpilogue ep) {
    const size_t total = (size_t)ep.R * ep.n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(e / ep.n), row = (uint32_t)(e % ep.n);
        // the splits' partial sums are loaded eight at a time (independent loads in flight)
        // and added in split order
        float acc = 0.f;
        const size_t stride = (size_t)ep.R * ep.n, at = (size_t)c * ep.n + row;
        for (uint32_t sp0 = 0; sp0 < ep.ksplit; sp0 += 8) {
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = sp0 + u < ep.ksplit ? ep.partial[(sp0 + u) * stride + at] : 0.f;
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (sp0 + u < ep.ksplit) acc += v[u];
        }
        if (ep.mode >= 2) {
            net_store(ep, row, c, acc);
            continue;
        }
        const float sc = ep.scale ? ep.scale[row] : 1.0f;
        float y = sc * acc;
        if (ep.mode == 1) {
            const float4 rh = ep.rho[row];
            const int ch = (int)(c % 3);
            const float rr = ch == 0 ? rh.x : (ch == 1 ? rh.y : rh.z);
            y = ep.resid[(size_t)c * ep.n + row] + rr * y;
        }
        ep.out[(size_t)c * ep.n + row] = y;
        if (ep.out16) ep.out16[(size_t)c * ep.ld16 + row] = __float2bfloat16_rn(ep.wscale ? y * ep.wscale[row] : y);
    }
}

// Split-K epilogue for many splits (the network's weight gradients): a warp per element, lane
// l adding splits l, l + 32, ... in order, then a fixed shuffle tree, so the sum is the same
// on every run.
__global__ void k_tc_finalize_wide(TcEpilogue ep) {
    const size_t total = (size_t)ep.R * ep.n;
    const uint32_t lane = threadIdx.x & 31;
    const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
    const size_t stride = (size_t)ep.R * ep.n;
    for (size_t e = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < total; e += warps) {
        const uint32_t c = (uint32_t)(e / ep.n), row = (uint32_t)(e % ep.n);
        const size_t at = (size_t)c * ep.n + row;
        float acc = 0.f;
        for (uint32_t sp = lane; sp < ep.ksplit; sp += 32) acc += ep.partial[sp * stride + at];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) net_store(ep, row, c, acc);
    }
}

uint32_t gemm_tc_width(uint32_t R);

// K splits for n rows and R right-hand sides: the count (1..8, at least 8 K blocks each)
// that minimises the bytes moved per row, with the F reads (2 ld bytes) divided by the
// share of the 152 SMs the last wave keeps busy, plus the partial sums written and read
// back (8 R bytes per split) when K is split.
uint32_t gemm_tc_ksplit(uint32_t n, uint32_t ld, uint32_t R) {
    const uint32_t rows = tc_mt(gemm_tc_width(R), 1) * kTcM;  // rows per CTA of the solve's sweeps
    const uint32_t tiles = (n + rows - 1) / rows, kblocks = ld / kTcBK;
    uint32_t best = 1;
    double best_cost = 1e300;
    for (uint32_t sp = 1; sp <= 8; sp++) {
        if (sp > 1 && kblocks / sp < 8) break;
        const double work = (double)tiles * sp;
        const double fill = work / (std::ceil(work / 152.0) * 152.0);
        const double cost = 2.0 * ld / fill + (sp > 1 ? 8.0 * R * sp : 0.0);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = sp;
        }
    }
    return best;
}

// Tensor maps by (base, rows, row length, box rows): a map depends on nothing else, so one
// encoded for a buffer is reused by every later launch on the same buffer and shape (the
// network's layers launch many small GEMMs, where encoding on the host per launch dominated).
struct MapKey {
    const void* base;
    uint64_t rows, ld;
    uint32_t box;
    bool operator==(const MapKey& o) const { return base == o.base && rows == o.rows && ld == o.ld && box == o.box; }
};
struct MapKeyHash {
    size_t operator()(const MapKey& k) const {
        uint64_t h = reinterpret_cast<uintptr_t>(k.base) * 0x9E3779B97F4A7C15ull;
        h ^= k.rows + 0x632BE59BD9B4E019ull + (h << 6) + (h >> 2);
        h ^= k.ld + 0x85EBCA77C2B2AE63ull + (h << 6) + (h >> 2);
        h ^= k.box + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

static bool cached_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t ld, uint32_t box_rows) {
    static std::mutex mu;
    static std::unordered_map<MapKey, CUtensorMap, MapKeyHash> cache;
    const MapKey key{base, rows, ld, box_rows};
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            *m = it->second;
            return true;
        }
    }
    if (!make_map(m, base, rows, ld, box_rows)) return false;
    std::lock_guard<std::mutex> lock(mu);
    if (cache.size() > 65536) cache.clear();
    cache.emplace(key, *m);
    return true;
}

template <int NR, int MT>
static int launch_tc_mt(const CUtensorMap& ma, const CUtensorMap& mb, uint32_t n, uint32_t kblocks,
                        const TcEpilogue& ep, cudaStream_t s) {
    using S = TcShape<NR, MT>;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_gemm_tc<NR, MT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem);
    if (attr != cudaSuccess) return -2;
    const uint32_t nsplit = (ep.partial && ep.ksplit > 1) ? ep.ksplit : 1u;
    const uint32_t per_split = (kblocks + nsplit - 1) / nsplit;  // K blocks of the longest split
    const uint32_t nst = per_split >= S::kMaxStages ? S::kMaxStages : (per_split < 2u ? 2u : per_split);
    const uint32_t tiles = (n + MT * kTcM - 1) / (MT * kTcM);
    k_gemm_tc<NR, MT><<<tiles * nsplit, 256, S::smem_for(nst), s>>>(ma, mb, kblocks, nst, ep);
    if (nsplit >= 32 && ep.mode >= 2) k_tc_finalize_wide<<<152 * 8, 256, 0, s>>>(ep);
    else if (nsplit > 1) k_tc_finalize<<<152 * 8, 256, 0, s>>>(ep);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

template <int NR>
static int launch_tc(const __nv_bfloat16* A, uint32_t n, uint32_t ld, const __nv_bfloat16* Bt, const TcEpilogue& ep,
                     cudaStream_t s) {
    CUtensorMap ma, mb;
    if (!cached_map(&ma, A, n, ld, kTcM) || !cached_map(&mb, Bt, NR, ld, NR)) return -1;
    const uint32_t kblocks = ld / kTcBK;
    if (tc_mt(NR, ep.mode) == 2) return launch_tc_mt<NR, 2>(ma, mb, n, kblocks, ep, s);
    return launch_tc_mt<NR, 1>(ma, mb, n, kblocks, ep, s);
}

// Shared-memory limits of the streaming residual and the tcgen05 GEMM instances, set before
// the first launch (and so before any stream capture that contains them).
cudaError_t dense_init() {
    cudaError_t e = resid_stream_init();
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sgemm_resid, cudaFuncAttributeMaxDynamicSharedMemorySize, kRSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<16, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<16, 1>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<32, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<32, 1>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<64, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<64, 1>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<128, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<128, 1>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<192, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<192, 1>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<256, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<256, 1>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<128, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<128, 2>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<192, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<192, 2>::kSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<256, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcShape<256, 2>::kSmem);
    return e;
}

// Bt must have Rpad = the template width rows (zero padded) and ld columns.
int launch_gemm_tc(const __nv_bfloat16* A, uint32_t n, uint32_t ld, const __nv_bfloat16* Bt, uint32_t Rpad,
                   const TcEpilogue& ep, cudaStream_t s) {
    switch (Rpad) {
        case 16: return launch_tc<16>(A, n, ld, Bt, ep, s);
        case 32: return launch_tc<32>(A, n, ld, Bt, ep, s);
        case 64: return launch_tc<64>(A, n, ld, Bt, ep, s);
        case 128: return launch_tc<128>(A, n, ld, Bt, ep, s);
        case 192: return launch_tc<192>(A, n, ld, Bt, ep, s);
        case 256: return launch_tc<256>(A, n, ld, Bt, ep, s);
        default: return -4;
    }
}

uint32_t gemm_tc_width(uint32_t R) {
    if (R <= 16) return 16;
    if (R <= 32) return 32;
    if (R <= 64) return 64;
    if (R <= 128) return 128;
    if (R <= 192) return 192;
    if (R <= 256) return 256;
    return 0;
}

}  // namespace rad
