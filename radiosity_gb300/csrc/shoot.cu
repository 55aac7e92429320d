// Shooting step on the device: shooter selection, radiosity update, emitter
// update and the stop rule (source/Main.cpp:1137-1303,
// source/ModelContainer.cpp:259-299).
//
// Selection (one CTA).  The reference keeps a std::list of at most K patch ids:
// patch 0 is always inserted; patch i>0 is inserted when |B_i|^2 > 0 and
// |B_i|^2 >= |B_back|^2, after which the list is stably sorted ascending,
// reversed, and truncated to K.  The sort + reverse flips the internal order of
// every group of equal energies at each insertion, so the final order depends on
// the insertion count.  This kernel reproduces it exactly: the list is stored in
// a canonical order in which the t-th insertion is placed at the front of its
// equal-energy group when t is even and at the back when t is odd, an eviction
// removes the canonical back (t even) or front (t odd) of the lowest group, and
// the output reverses each group when the final insertion count is odd.
// Patches are streamed in index order in chunks of 4096; a chunk's candidates
// (E > 0 and E >= the list minimum at chunk start, a superset of the inserted
// ones) are compacted in index order and inserted by warp 0.
// PHYS mode selects the K largest unshot powers (r+g+b)*A, ties to lower index.
#include <cuda_runtime.h>
#include <stdint.h>

#include "rad_internal.cuh"

namespace rad {

constexpr int kSelThreads = 1024;
constexpr int kChunk = 4096;

__device__ __forceinline__ float sel_value(int mode, float4 r, float a) {
    if (mode == 0) return r.x * r.x + r.y * r.y + r.z * r.z;  // Vector3::f_Length2
    return ((r.x + r.y) + r.z) * a;
}

// warp 0 helpers over the list (lv, li, size n) in shared memory
__device__ __forceinline__ int warp_count(const float* lv, int n, float v, bool ge) {
    const int lane = threadIdx.x & 31;
    int c = 0;
    for (int j = lane; j < n; j += 32) c += ge ? (lv[j] >= v) : (lv[j] > v);
    return (int)__reduce_add_sync(0xffffffffu, (unsigned)c);
}

__device__ __forceinline__ void warp_shift_right(float* lv, uint32_t* li, int pos, int n) {
    const int lane = threadIdx.x & 31;
    for (int top = n - 1; top >= pos; top -= 32) {
        const int j = top - lane;
        const bool ok = j >= pos;
        float v = 0;
        uint32_t id = 0;
        if (ok) {
            v = lv[j];
            id = li[j];
        }
        __syncwarp();
        if (ok) {
            lv[j + 1] = v;
            li[j + 1] = id;
        }
        __syncwarp();
    }
}

__device__ __forceinline__ void warp_shift_left(float* lv, uint32_t* li, int rm, int n) {
    const int lane = threadIdx.x & 31;
    for (int lo = rm + 1; lo < n; lo += 32) {
        const int j = lo + lane;
        const bool ok = j < n;
        float v = 0;
        uint32_t id = 0;
        if (ok) {
            v = lv[j];
            id = li[j];
        }
        __syncwarp();
        if (ok) {
            lv[j - 1] = v;
            li[j - 1] = id;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kSelThreads) k_select(Geo g, Batch b, const float4* __restrict__ rad,
                                                        const float* __restrict__ area, DevState* st) {
    if (st->stopped) return;
    const int mode = (int)g.mode;
    const int K = (int)b.K;
    const uint32_t N = g.n;
    __shared__ float lv[kMaxK + 1];
    __shared__ uint32_t li[kMaxK + 1];
    __shared__ float pv[kChunk];
    __shared__ uint32_t pi[kChunk];
    __shared__ uint32_t wcount[32];
    __shared__ int s_n, s_t, s_pc;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t start = 0;
    if (tid == 0) {
        s_pc = 0;
        if (mode == 0) {  // tops.empty(): patch 0 always enters
            lv[0] = sel_value(0, rad[0], 0.f);
            li[0] = 0;
            s_n = 1;
            s_t = 1;
        } else {
            s_n = 0;
            s_t = 0;
        }
    }
    if (mode == 0) start = 1;
    __syncthreads();
    for (uint32_t base = start; base < N; base += kChunk) {
        const int n0 = s_n;
        const float thr = n0 > 0 ? lv[n0 - 1] : 0.f;
        const bool full = n0 >= K;
        for (int sub = 0; sub < kChunk / kSelThreads; sub++) {
            const uint32_t j = base + sub * kSelThreads + tid;
            bool pot = false;
            float v = 0;
            if (j < N) {
                v = sel_value(mode, rad[j], mode ? area[j] : 0.f);
                if (mode == 0) pot = v > 0 && v >= thr;
                else pot = v > 0 && (!full || v > thr);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, pot);
            if (lane == 0) wcount[warp] = __popc(bal);
            __syncthreads();
            if (warp == 0) {
                uint32_t c = wcount[lane], x = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                wcount[lane] = x - c;  // exclusive prefix
            }
            __syncthreads();
            if (pot) {
                const int pos = s_pc + (int)wcount[warp] + __popc(bal & ((1u << lane) - 1u));
                pv[pos] = v;
                pi[pos] = j;
            }
            __syncthreads();
            // the last lane of the last warp knows the chunk total
            if (warp == 31 && lane == 31) s_pc += (int)wcount[31] + __popc(bal);
            __syncthreads();
        }
        if (warp == 0) {
            int n = s_n, t = s_t;
            const int pc = s_pc;
            for (int i = 0; i < pc; i++) {
                const float v = pv[i];
                const uint32_t id = pi[i];
                if (mode == 0) {
                    if (!(v >= lv[n - 1])) continue;
                    t++;
                    const int gs = warp_count(lv, n, v, false), ge = warp_count(lv, n, v, true);
                    const int pos = (t & 1) ? ge : gs;
                    warp_shift_right(lv, li, pos, n);
                    if (lane == 0) {
                        lv[pos] = v;
                        li[pos] = id;
                    }
                    __syncwarp();
                    n++;
                    if (n > K) {
                        const float low = lv[n - 1];
                        const int ls = warp_count(lv, n, low, false);
                        const int rm = (t & 1) ? ls : n - 1;
                        warp_shift_left(lv, li, rm, n);
                        n--;
                    }
                } else {
                    if (n >= K && !(v > lv[n - 1])) continue;
                    const int pos = warp_count(lv, n, v, true);
                    warp_shift_right(lv, li, pos, n);
                    if (lane == 0) {
                        lv[pos] = v;
                        li[pos] = id;
                    }
                    __syncwarp();
                    n++;
                    if (n > K) n = K;
                }
            }
            if (lane == 0) {
                s_n = n;
                s_t = t;
                s_pc = 0;
            }
        }
        __syncthreads();
    }
    // output
    const int n = s_n;
    const bool flip = mode == 0 && (s_t & 1);
    for (int j = tid; j < K; j += blockDim.x) {
        if (j >= n) {
            b.shooters[j] = 0;
            b.valid[j] = 0;
        }
    }
    for (int j = tid; j < n; j += blockDim.x) {
        int out = j;
        if (flip) {
            const float v = lv[j];
            int gs = 0, ge = 0;
            for (int k = 0; k < n; k++) {
                gs += lv[k] > v;
                ge += lv[k] >= v;
            }
            out = gs + ge - 1 - j;
        }
        b.shooters[out] = li[j];
        b.valid[out] = 1;
    }
}

// ---------------------------------------------------------------------------
// PHYS selection: K largest unshot powers, ties to the lower index.  Keys are the
// float bits of the power (monotonic for positives); composites
// (key << 32 | ~index) are unique and order exactly as required.  A 2048-bin
// histogram of the top 12 key bits finds the boundary bin; elements above it
// are selected outright, the boundary bin is refined by an exact radix select
// on the composites in one CTA, and the K winners are bitonic-sorted.
// ---------------------------------------------------------------------------
constexpr int kHist = 2048;

__global__ void __launch_bounds__(256) k_psel_hist(Geo g, Batch b, const float4* __restrict__ rad,
                                                   const float* __restrict__ area, DevState* st) {
    if (st->stopped) return;
    __shared__ uint32_t h[kHist];
    for (int i = threadIdx.x; i < kHist; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const float v = sel_value(1, rad[i], area[i]);
        const uint32_t bits = v > 0 ? __float_as_uint(v) : 0u;
        b.sel_keys[i] = bits;
        if (bits) atomicAdd(&h[bits >> 20], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHist; i += blockDim.x)
        if (h[i]) atomicAdd(&b.sel_hist[i], h[i]);
}

__global__ void __launch_bounds__(1024) k_psel_pick(Batch b, DevState* st) {
    if (st->stopped) return;
    __shared__ uint32_t suf[kHist + 1];
    __shared__ uint32_t part[1024];
    const int t = threadIdx.x;
    // suffix sums: element r of the reversed histogram is bin kHist-1-r
    const uint32_t a0 = b.sel_hist[kHist - 1 - 2 * t], a1 = b.sel_hist[kHist - 2 - 2 * t];
    part[t] = a0 + a1;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    const uint32_t before = part[t] - (a0 + a1);
    suf[kHist - 1 - 2 * t] = before + a0;
    suf[kHist - 2 - 2 * t] = before + a0 + a1;
    if (t == 0) suf[kHist] = 0;
    __syncthreads();
    const uint32_t K = b.K, total = suf[0];
    for (int i = t; i < kHist; i += blockDim.x) {
        const bool pick = total < K ? (i == 0) : (suf[i] >= K && suf[i + 1] < K);
        if (pick) {
            b.sel_ctrl[0] = (uint32_t)i;
            b.sel_ctrl[1] = suf[i + 1];
        }
    }
    if (t == 0) {
        b.sel_ctrl[2] = 0;
        b.sel_ctrl[3] = 0;
        b.sel_ctrl[4] = total;
    }
    __syncthreads();
    for (int i = t; i < kHist; i += blockDim.x) b.sel_hist[i] = 0;  // ready for the next batch
}

__global__ void __launch_bounds__(256) k_psel_collect(Geo g, Batch b, DevState* st) {
    if (st->stopped) return;
    const uint32_t B = b.sel_ctrl[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const uint32_t bits = b.sel_keys[i];
        if (!bits) continue;
        const uint32_t bin = bits >> 20;
        if (bin < B) continue;
        const unsigned long long comp = ((unsigned long long)bits << 32) | (0xFFFFFFFFu - i);
        if (bin > B) {
            const uint32_t pos = atomicAdd(&b.sel_ctrl[2], 1u);
            if (pos < b.K) b.sel_sure[pos] = comp;
        } else {
            const uint32_t pos = atomicAdd(&b.sel_ctrl[3], 1u);
            if (pos < g.n) b.sel_bnd[pos] = comp;
        }
    }
}

__global__ void __launch_bounds__(1024) k_psel_final(Geo g, Batch b, DevState* st) {
    if (st->stopped) return;
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long arr[kMaxK];
    __shared__ unsigned long long s_prefix, s_mask;
    __shared__ uint32_t s_rem, s_cnt, s_done;
    const int t = threadIdx.x;
    const uint32_t K = b.K, n_sure = min(b.sel_ctrl[2], K), n_bnd = min(b.sel_ctrl[3], g.n);
    const uint32_t take = min(K, b.sel_ctrl[4]);
    const uint32_t R = take > n_sure ? take - n_sure : 0u;
    if (t == 0) {
        s_prefix = 0;
        s_mask = 0;
        s_rem = R;
        s_cnt = 0;
        s_done = 0;
    }
    __syncthreads();
    // Boundary elements share the top 12 composite bits (their histogram bin); an
    // exact radix select over the low 52 bits (digits of 8,8,8,8,8,8,4 bits) finds
    // the R-th largest composite, so exactly R boundary elements are >= thr.
    unsigned long long thr = 0;
    if (R < n_bnd) {
        const int shifts[7] = {44, 36, 28, 20, 12, 4, 0};
        for (int d = 0; d < 7; d++) {
            const int sh = shifts[d];
            const unsigned long long dmask = d < 6 ? 0xFFull : 0xFull;
            for (int i = t; i < 256; i += blockDim.x) hist[i] = 0;
            __syncthreads();
            const unsigned long long pm = s_mask, pv = s_prefix;
            for (uint32_t j = t; j < n_bnd; j += blockDim.x) {
                const unsigned long long c = b.sel_bnd[j];
                if ((c & pm) == pv) atomicAdd(&hist[(c >> sh) & dmask], 1u);
            }
            __syncthreads();
            if (t < 32) {
                // the bin holding the rem-th largest: lane l covers bins dmask - 8l .. dmask - 8l - 7
                // (descending); a warp scan of the lanes' totals finds the lane, which walks its bins
                const uint32_t rem = s_rem;
                const int top = (int)dmask - 8 * t;
                uint32_t local = 0;
                for (int j = 0; j < 8; j++)
                    if (top - j >= 0) local += hist[top - j];
                uint32_t incl = local;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (t >= o) incl += y;
                }
                const uint32_t excl = incl - local;
                if (excl < rem && rem <= incl) {
                    uint32_t cum = excl;
                    for (int j = 0; j < 8; j++) {
                        const int v = top - j;
                        if (cum + hist[v] >= rem) {
                            s_rem = rem - cum;
                            s_prefix = pv | ((unsigned long long)v << sh);
                            s_mask = pm | (dmask << sh);
                            // the bin is taken whole: the prefix with zero low digits is the
                            // threshold that selects exactly rem elements
                            s_done = cum + hist[v] == rem ? 1u : 0u;
                            break;
                        }
                        cum += hist[v];
                    }
                }
            }
            __syncthreads();
            if (s_done) break;
        }
        thr = s_prefix;
    }
    // gather the winners
    for (uint32_t j = t; j < n_sure; j += blockDim.x) arr[j] = b.sel_sure[j];
    __syncthreads();
    const unsigned long long lowmask = 0x000FFFFFFFFFFFFFull;
    for (uint32_t j = t; j < n_bnd; j += blockDim.x) {
        const unsigned long long c = b.sel_bnd[j];
        if (R >= n_bnd || (c & lowmask) >= thr) {
            const uint32_t pos = n_sure + atomicAdd(&s_cnt, 1u);
            if (pos < K) arr[pos] = c;
        }
    }
    __syncthreads();
    uint32_t P = 32;
    while (P < take) P <<= 1;
    for (uint32_t j = take + t; j < P; j += blockDim.x) arr[j] = 0;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = t; i < P; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = arr[i], c = arr[ixj];
                    const bool desc = (i & k) == 0;
                    if (desc ? (a < c) : (a > c)) {
                        arr[i] = c;
                        arr[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (uint32_t k = t; k < K; k += blockDim.x) {
        if (k < take) {
            b.shooters[k] = 0xFFFFFFFFu - (uint32_t)(arr[k] & 0xFFFFFFFFull);
            b.valid[k] = 1;
        } else {
            b.shooters[k] = 0;
            b.valid[k] = 0;
        }
    }
}

void launch_select(const Geo& g, const Batch& b, const float4* rad, const float* area, DevState* st,
                   cudaStream_t s) {
    if (g.mode == 0) {
        k_select<<<1, kSelThreads, 0, s>>>(g, b, rad, area, st);
        return;
    }
    uint32_t blocks = (g.n + 255) / 256;
    if (blocks > 152 * 4) blocks = 152 * 4;
    k_psel_hist<<<blocks, 256, 0, s>>>(g, b, rad, area, st);
    k_psel_pick<<<1, 1024, 0, s>>>(b, st);
    k_psel_collect<<<blocks, 256, 0, s>>>(g, b, st);
    k_psel_final<<<1, 1024, 0, s>>>(g, b, st);
}

// ---------------------------------------------------------------------------
// Radiosity update (source/Main.cpp:1271-1278)
// ---------------------------------------------------------------------------
constexpr int kUpdateThreads = 128;  // small blocks: 4 per SM even at N = 50k
__global__ void __launch_bounds__(kUpdateThreads) k_update(Geo g, Batch b, const float4* __restrict__ color,
                                                const float4* __restrict__ rho, const float* __restrict__ area,
                                                float4* __restrict__ rad, DevState* st) {
    if (st->stopped) return;
    const int K = (int)b.K;
    __shared__ float4 s_saved[kMaxK];
    __shared__ float4 s_col[kMaxK];
    __shared__ float s_area[kMaxK];
    __shared__ uint32_t s_valid[kMaxK];
    for (int h = threadIdx.x; h < K; h += blockDim.x) {
        const uint32_t v = b.valid[h];
        s_valid[h] = v;
        if (v) {
            const uint32_t e = b.shooters[h];
            s_saved[h] = b.saved[h];
            s_col[h] = color[e];
            s_area[h] = g.mode ? area[e] : 0.f;
        }
    }
    __syncthreads();
    const uint32_t N = g.n;
    double acc = 0;
    // The hemicubes' contributions are added in hemicube order (the float sums must match
    // the oracle's order); their exact sums are loaded kLoad at a time ahead of use, so a
    // thread keeps several independent loads in flight instead of one.
    constexpr int kLoad = 16;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        float4 r = rad[i];
        const float ai = g.mode ? area[i] : 0.f;
        const float4 rh = g.mode ? rho[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int h0 = 0; h0 < K; h0 += kLoad) {
            unsigned long long qv[kLoad];
#pragma unroll
            for (int j = 0; j < kLoad; j++) {
                const int h = h0 + j;
                qv[j] = (h < K && s_valid[h]) ? b.Fq[(size_t)h * N + i] : 0ull;
            }
#pragma unroll
            for (int j = 0; j < kLoad; j++) {
                const unsigned long long q = qv[j];
                if (q == 0) continue;
                const int h = h0 + j;
                b.Fq[(size_t)h * N + i] = 0;  // ready for the next batch
                const float F = __ull2float_rn(q) * 0x1p-61f;
                const float4 sv = s_saved[h];
                float t;
                if (g.mode == 0) {  // source/Main.cpp:1274, REFLECTIVITY and the shooter's colour
                    const float4 c = s_col[h];
                    t = sv.x * F; t = t * kReflectivity; t = t * c.x; r.x = r.x + t;
                    t = sv.y * F; t = t * kReflectivity; t = t * c.y; r.y = r.y + t;
                    t = sv.z * F; t = t * kReflectivity; t = t * c.z; r.z = r.z + t;
                } else {
                    if (!(ai > 0)) continue;
                    const float gg = (F * s_area[h]) / ai;
                    t = sv.x * gg; t = rh.x * t; r.x = r.x + t;
                    t = sv.y * gg; t = rh.y * t; r.y = r.y + t;
                    t = sv.z * gg; t = rh.z * t; r.z = r.z + t;
                }
            }
        }
        rad[i] = r;
        if (g.mode != 0) acc += (double)area[i] * (((double)r.x + (double)r.y) + (double)r.z);
    }
    if (g.mode != 0) {  // FP64 partial of the unshot power after the update (residual)
        __shared__ double red[kUpdateThreads];
        red[threadIdx.x] = acc;
        __syncthreads();
        for (uint32_t o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) b.partials[blockIdx.x] = red[0];
    }
}

static uint32_t update_blocks(uint32_t n) {
    uint32_t blocks = (n + kUpdateThreads - 1) / kUpdateThreads;
    if (blocks > (uint32_t)kUpdateBlocks) blocks = kUpdateBlocks;
    return blocks ? blocks : 1;
}

void launch_update(const Geo& g, const Batch& b, const float4* color, const float4* rho, const float* area,
                   float4* rad, DevState* st, cudaStream_t s) {
    k_update<<<update_blocks(g.n), kUpdateThreads, 0, s>>>(g, b, color, rho, area, rad, st);
}

// ---------------------------------------------------------------------------
// Emitters + stop rule (source/Main.cpp:1286-1303); PHYS residual in FP64
// ---------------------------------------------------------------------------
__device__ double block_unshot_power(const float4* __restrict__ rad, const float* __restrict__ area, uint32_t n,
                                     double* red) {
    double s = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 r = rad[i];
        s += (double)area[i] * ((double)r.x + (double)r.y + (double)r.z);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// Emitters of one batch are distinct patches, so their updates run in parallel;
// lastEnergy is the pre-subtraction radiosity of the last valid emitter.
__global__ void __launch_bounds__(256) k_emitters(Geo g, Batch b, float4* __restrict__ rad,
                                                  float4* __restrict__ illum, const float* __restrict__ area,
                                                  double tol, uint32_t nparts, DevState* st) {
    if (st->stopped) return;
    __shared__ double red[256];
    __shared__ int s_last;
    __shared__ uint32_t s_nv;
    if (threadIdx.x == 0) {
        s_last = -1;
        s_nv = 0;
    }
    __syncthreads();
    uint32_t nv = 0;
    for (uint32_t h = threadIdx.x; h < b.K; h += blockDim.x)
        if (b.valid[h]) {
            atomicMax(&s_last, (int)h);
            nv++;
        }
    atomicAdd(&s_nv, nv);
    __syncthreads();
    const int last = s_last;
    double corr = 0;
    for (uint32_t h = threadIdx.x; h < b.K; h += blockDim.x) {
        if (!b.valid[h]) continue;
        const uint32_t e = b.shooters[h];
        float4 r = rad[e], il = illum[e];
        const float4 sv = b.saved[h];
        if ((int)h == last) {
            st->last_energy[0] = r.x;
            st->last_energy[1] = r.y;
            st->last_energy[2] = r.z;
            if (g.mode == 0) {
                const bool stop = (double)sqrtf(r.x * r.x + r.y * r.y + r.z * r.z) < 0.1;
                if (stop) st->stopped = 1;
            }
        }
        if (g.mode != 0) corr -= (double)area[e] * (((double)r.x + (double)r.y) + (double)r.z);
        il.x = il.x + sv.x; il.y = il.y + sv.y; il.z = il.z + sv.z;
        r.x = r.x - sv.x; r.y = r.y - sv.y; r.z = r.z - sv.z;
        if (g.mode != 0) corr += (double)area[e] * (((double)r.x + (double)r.y) + (double)r.z);
        rad[e] = r;
        illum[e] = il;
    }
    if (threadIdx.x == 0) {
        st->shots_done += 1;
        st->hemicubes += (double)s_nv;
    }
    if (g.mode != 0) {
        double p = corr;
        for (uint32_t i = threadIdx.x; i < nparts; i += blockDim.x) p += b.partials[i];
        red[threadIdx.x] = p;
        __syncthreads();
        for (uint32_t o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const double res = st->power0 > 0 ? red[0] / st->power0 : 0.0;
            st->residual = res;
            if (res <= tol) st->stopped = 1;
        }
    }
}

__global__ void __launch_bounds__(256) k_power0(const float4* __restrict__ rad, const float* __restrict__ area,
                                                uint32_t n, DevState* st) {
    __shared__ double red[256];
    const double p = block_unshot_power(rad, area, n, red);
    if (threadIdx.x == 0) {
        st->power0 = p;
        st->residual = p > 0 ? 1.0 : 0.0;
    }
}

void launch_emitters(const Geo& g, const Batch& b, float4* rad, float4* illum, const float* area, double tol,
                     double* partials, DevState* st, cudaStream_t s) {
    (void)partials;
    k_emitters<<<1, 256, 0, s>>>(g, b, rad, illum, area, tol, update_blocks(g.n), st);
}

void launch_power0(const float4* rad, const float* area, uint32_t n, DevState* st, cudaStream_t s) {
    k_power0<<<1, 256, 0, s>>>(rad, area, n, st);
}

// Quad areas for PHYS mode: 0.5*|(v1-v3) x (v2-v4)|.
__global__ void k_areas(const float* __restrict__ verts, uint32_t n, float* __restrict__ area) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* q = verts + 12 * (size_t)p;
    const float ax = q[0] - q[6], ay = q[1] - q[7], az = q[2] - q[8];
    const float bx = q[3] - q[9], by = q[4] - q[10], bz = q[5] - q[11];
    const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    area[p] = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
}

void launch_areas(const float* verts, uint32_t n, float* area, cudaStream_t s) {
    k_areas<<<(n + 255) / 256, 256, 0, s>>>(verts, n, area);
}

// The host's per-patch float3 arrays (ModelContainer's AoS layout) arrive by one DMA into a
// device scratch and are widened here to the solver's float4 rows (w = 0), and back.
__global__ void k_f3_to_f4(const float* __restrict__ src, float4* __restrict__ dst, uint32_t n) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        dst[p] = make_float4(src[3 * (size_t)p], src[3 * (size_t)p + 1], src[3 * (size_t)p + 2], 0.f);
}

__global__ void k_f4_to_f3(const float4* __restrict__ src, float* __restrict__ dst, uint32_t n) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const float4 v = src[p];
        dst[3 * (size_t)p] = v.x;
        dst[3 * (size_t)p + 1] = v.y;
        dst[3 * (size_t)p + 2] = v.z;
    }
}

void launch_f3_to_f4(const float* src, float4* dst, uint32_t n, cudaStream_t s) {
    k_f3_to_f4<<<152 * 4, 256, 0, s>>>(src, dst, n);
}

void launch_f4_to_f3(const float4* src, float* dst, uint32_t n, cudaStream_t s) {
    k_f4_to_f3<<<152 * 4, 256, 0, s>>>(src, dst, n);
}

}  // namespace rad
