// The narrow FP32 residual of the gathering solve (R <= 4 right-hand sides), in its own
// translation unit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "rad_internal.cuh"
#include "pipe.cuh"

namespace rad {

// ---------------------------------------------------------------------------
// Narrow residual, R <= 4 right-hand sides (one scene's RGB solve).  The product is then a
// stream over F with little arithmetic (the tiled 128x64 kernel of dense.cu would issue 16x
// its useful FMAs), so the kernel is built to keep HBM busy.  A CTA owns 16 rows.  One producer warp
// moves F through a 3-stage shared-memory ring with 1-D bulk copies (cp.async.bulk, one
// 2-KB row segment per lane, completion counted in bytes on the stage's mbarrier), so
// ~96 KB per CTA are in flight without holding registers.  Eight consumer warps take 2 rows
// each: lane l reads columns 4l + 128j of the stage from shared memory (conflict-free float4)
// and the right-hand sides from a zero-padded copy with row pitch ld (float4 through L1, the
// same addresses for all warps of the CTA).  Partial sums (16 terms) are folded into a
// (hi, lo) TwoSum pair after each stage and the lanes' pairs are combined by a TwoSum
// butterfly, keeping the wide kernel's compensated accuracy.  Columns >= n of F (row
// padding, never written) are masked to zero before use.  Every wait is bounded (kWaitNs);
// a timeout sets *err and the warp stops.  Instantiated for 3 slots (R <= 3, one scene's RGB)
// and 4: every slot costs loads and FMAs.  On a 50k-patch scene with R = 3 one residual
// streams its 10.2 GB of F at about 0.9 of the measured HBM copy bandwidth.
// ---------------------------------------------------------------------------
constexpr int kNR = 4;                       // right-hand-side slots
static_assert(kNR == (int)kResidStreamRhs, "the slots of the scratch sizing");
constexpr int kNRows = 16;                   // rows per CTA
constexpr int kNCols = 512;                  // columns per stage
constexpr int kNStages = 3;
constexpr int kNConsumers = 8;               // consumer warps (2 rows each)
constexpr int kNHoist = 2;                   // 128-column slices whose loads are issued together
constexpr int kNStageBytes = kNRows * kNCols * 4;  // 32 KB
constexpr int kNSmem = kNStages * kNStageBytes + 2 * kNStages * 8;

// Xp[c][k] = X[c][k] for c < R, k < n, else 0; Xp has kNR rows of pitch ld.
// With weights w: Xp[c][k] = w[k] * X[c][k].
__global__ void k_pad_rhs(const float* __restrict__ X, uint32_t n, uint32_t R, uint32_t ld, float* __restrict__ Xp,
                          const float* __restrict__ w) {
    const size_t total = (size_t)kNR * ld;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(t / ld), k = (uint32_t)(t % ld);
        Xp[t] = (c < R && k < n) ? X[(size_t)c * n + k] * (w ? w[k] : 1.0f) : 0.f;
    }
}

// (hi, lo) += b with Knuth's TwoSum: the rounding error of hi + b goes to lo.
__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float b) {
    const float s = hi + b, bv = s - hi;
    lo += (hi - (s - bv)) + (b - bv);
    hi = s;
}

__device__ __forceinline__ void fma4(float& a, const float4& f, const float4& x) {
    a = fmaf(f.x, x.x, a);
    a = fmaf(f.y, x.y, a);
    a = fmaf(f.z, x.z, a);
    a = fmaf(f.w, x.w, a);
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

template <int NRC>
__global__ void __launch_bounds__((kNConsumers + 1) * 32, 2)
    k_resid_stream(const float* __restrict__ F, uint32_t n, uint32_t ld, const float* __restrict__ Xp,
                   const float* __restrict__ X, const float* __restrict__ E, const float4* __restrict__ rho,
                   uint32_t R, float* r, double* nrm, uint32_t* err, const float* __restrict__ inv_a) {
    extern __shared__ __align__(128) uint8_t s_raw[];
    float* stage = reinterpret_cast<float*>(s_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(s_raw + kNStages * kNStageBytes);
    uint64_t* empty = full + kNStages;
    __shared__ double s_nrm[kNConsumers][kNR];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t row0 = blockIdx.x * kNRows;
    const uint32_t nst = (n + kNCols - 1) / kNCols;
    if (threadIdx.x == 0) {
        for (int i = 0; i < kNStages; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], kNConsumers);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == kNConsumers) {
        // producer: stage t gets columns [t*512, t*512 + 512) of the CTA's rows
        const uint32_t nrows = min((uint32_t)kNRows, n - row0);
        for (uint32_t t = 0; t < nst; t++) {
            const uint32_t sidx = t % kNStages, round = t / kNStages;
            bool ok = true;
            if (lane == 0) ok = mbar_wait(&empty[sidx], (round & 1u) ^ 1u, err);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            const uint32_t k = t * kNCols, bytes = 4u * min((uint32_t)kNCols, ld - k);  // multiple of 256 B
            if (lane == 0) mbar_expect_tx(&full[sidx], bytes * nrows);
            __syncwarp();
            if ((uint32_t)lane < nrows)
                bulk_load(stage + (size_t)sidx * (kNStageBytes / 4) + lane * kNCols, F + (size_t)(row0 + lane) * ld + k,
                          bytes, &full[sidx]);
        }
    } else {
        const int pr0 = warp * 2;  // the warp's rows within the CTA
        float acc[2][NRC], hi[2][NRC], lo[2][NRC];
#pragma unroll
        for (int p = 0; p < 2; p++)
#pragma unroll
            for (int c = 0; c < NRC; c++) acc[p][c] = hi[p][c] = lo[p][c] = 0.f;
        const float4* X4 = reinterpret_cast<const float4*>(Xp);
        const uint32_t ld4 = ld / 4;
        const bool rv0 = row0 + pr0 < n, rv1 = row0 + pr0 + 1 < n;
        for (uint32_t t = 0; t < nst; t++) {
            const uint32_t sidx = t % kNStages, round = t / kNStages;
            bool ok = true;
            if (lane == 0) ok = mbar_wait(&full[sidx], round & 1u, err);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            const float* st = stage + (size_t)sidx * (kNStageBytes / 4);
            const uint32_t k0 = t * kNCols;
            // two 128-column slices at a time: all their loads are issued before the FMAs, so
            // the shared-memory and L1 latencies overlap (columns >= n load nothing and add 0)
#pragma unroll
            for (int jh = 0; jh < kNCols / 128; jh += kNHoist) {
                float4 f0[kNHoist], f1[kNHoist], x[kNHoist][NRC];
#pragma unroll
                for (int j = 0; j < kNHoist; j++) {
                    const uint32_t col = (uint32_t)(lane * 4 + (jh + j) * 128), k = k0 + col;
                    const bool in = k < n;
                    f0[j] = (in && rv0) ? *reinterpret_cast<const float4*>(st + pr0 * kNCols + col)
                                        : make_float4(0, 0, 0, 0);
                    f1[j] = (in && rv1) ? *reinterpret_cast<const float4*>(st + (pr0 + 1) * kNCols + col)
                                        : make_float4(0, 0, 0, 0);
#pragma unroll
                    for (int c = 0; c < NRC; c++)  // k < n <= ld - 3 keeps the read inside Xp
                        x[j][c] = in ? __ldg(X4 + (size_t)c * ld4 + k / 4) : make_float4(0, 0, 0, 0);
                    if (in && k + 4 > n) {  // the row padding beyond n is not data
                        if (k + 1 >= n) f0[j].y = f1[j].y = 0.f;
                        if (k + 2 >= n) f0[j].z = f1[j].z = 0.f;
                        f0[j].w = f1[j].w = 0.f;
                    }
                }
#pragma unroll
                for (int j = 0; j < kNHoist; j++)
#pragma unroll
                    for (int c = 0; c < NRC; c++) {
                        fma4(acc[0][c], f0[j], x[j][c]);
                        fma4(acc[1][c], f1[j], x[j][c]);
                    }
            }
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&empty[sidx])) : "memory");
#pragma unroll
            for (int p = 0; p < 2; p++)
#pragma unroll
                for (int c = 0; c < NRC; c++) {
                    two_sum_add(hi[p][c], lo[p][c], acc[p][c]);
                    acc[p][c] = 0.f;
                }
        }
        // lanes' (hi, lo) pairs -> one pair per (row, column), the same in every lane
        float mine = 0.f;
#pragma unroll
        for (int p = 0; p < 2; p++)
#pragma unroll
            for (int c = 0; c < NRC; c++) {
                float h = hi[p][c], l = lo[p][c];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float h2 = __shfl_xor_sync(0xffffffffu, h, o), l2 = __shfl_xor_sync(0xffffffffu, l, o);
                    const float s2 = h + h2, bv = s2 - h;
                    l = (l + l2) + ((h - (s2 - bv)) + (h2 - bv));
                    h = s2;
                }
                if (lane == p * kNR + c) mine = h + l;
            }
        // lane p*4 + c writes row row0 + pr0 + p, column c
        const int p = lane / kNR, c = lane % kNR;
        double sq = 0.0;
        if (lane < 2 * kNR && (uint32_t)c < R && row0 + pr0 + p < n) {
            const uint32_t i = row0 + pr0 + p;
            const float4 rh = rho[i];
            const int chn = c % 3;
            const float rr = chn == 0 ? rh.x : (chn == 1 ? rh.y : rh.z);
            const float v = E[(size_t)c * n + i] + rr * (mine * (inv_a ? inv_a[i] : 1.0f)) - X[(size_t)c * n + i];
            r[(size_t)c * n + i] = v;
            sq = (double)v * (double)v;
        }
        sq += __shfl_xor_sync(0xffffffffu, sq, 4);
        if (lane < kNR) s_nrm[warp][lane] = sq;
    }
    __syncthreads();
    if (nrm && threadIdx.x < R) {
        double t = 0.0;
        for (int w = 0; w < kNConsumers; w++) t += s_nrm[w][threadIdx.x];
        atomicAdd(&nrm[threadIdx.x], t);
    }
}

void launch_resid_stream(const float* F, uint32_t n, uint32_t ld, const float* X, const float* E, const float4* rho,
                         uint32_t R, float* r, double* nrm, float* scratch, uint32_t* err, cudaStream_t s,
                         const float* w, const float* inv_a) {
    k_pad_rhs<<<152 * 2, 256, 0, s>>>(X, n, R, ld, scratch, w);
    const dim3 grid((n + kNRows - 1) / kNRows), block((kNConsumers + 1) * 32);
    if (R <= 3) k_resid_stream<3><<<grid, block, kNSmem, s>>>(F, n, ld, scratch, X, E, rho, R, r, nrm, err, inv_a);
    else k_resid_stream<4><<<grid, block, kNSmem, s>>>(F, n, ld, scratch, X, E, rho, R, r, nrm, err, inv_a);
}

cudaError_t resid_stream_init() {
    cudaError_t e = cudaFuncSetAttribute(k_resid_stream<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_resid_stream<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNSmem);
    return e;
}

}  // namespace rad
