// Shooting step on the device: shooter selection, radiosity update, emitter
// update and the stop rule (source/Main.cpp:1137-1303,
// source/ModelContainer.cpp:313-353).
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

void launch_select(const Geo& g, const Batch& b, const float4* rad, const float* area, DevState* st,
                   cudaStream_t s) {
    k_select<<<1, kSelThreads, 0, s>>>(g, b, rad, area, st);
}

// ---------------------------------------------------------------------------
// Radiosity update (source/Main.cpp:1271-1278)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_update(Geo g, Batch b, const float4* __restrict__ color,
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
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        float4 r = rad[i];
        if (g.mode == 0) {
            for (int h = 0; h < K; h++) {
                if (!s_valid[h]) continue;
                unsigned long long* fq = b.Fq + (size_t)h * N + i;
                const unsigned long long q = *fq;
                if (q == 0) continue;
                *fq = 0;
                const float F = __ull2float_rn(q) * 0x1p-61f;
                const float4 s = s_saved[h], c = s_col[h];
                float t;
                t = s.x * F; t = t * kReflectivity; t = t * c.x; r.x = r.x + t;
                t = s.y * F; t = t * kReflectivity; t = t * c.y; r.y = r.y + t;
                t = s.z * F; t = t * kReflectivity; t = t * c.z; r.z = r.z + t;
            }
        } else {
            const float ai = area[i];
            const float4 rh = rho[i];
            for (int h = 0; h < K; h++) {
                if (!s_valid[h]) continue;
                unsigned long long* fq = b.Fq + (size_t)h * N + i;
                const unsigned long long q = *fq;
                if (q == 0) continue;
                *fq = 0;
                if (!(ai > 0)) continue;
                const float F = __ull2float_rn(q) * 0x1p-61f;
                const float gg = (F * s_area[h]) / ai;
                const float4 s = s_saved[h];
                float t;
                t = s.x * gg; t = rh.x * t; r.x = r.x + t;
                t = s.y * gg; t = rh.y * t; r.y = r.y + t;
                t = s.z * gg; t = rh.z * t; r.z = r.z + t;
            }
        }
        rad[i] = r;
    }
}

void launch_update(const Geo& g, const Batch& b, const float4* color, const float4* rho, const float* area,
                   float4* rad, DevState* st, cudaStream_t s) {
    uint32_t blocks = (g.n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks == 0) blocks = 1;
    k_update<<<blocks, 256, 0, s>>>(g, b, color, rho, area, rad, st);
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

__global__ void __launch_bounds__(256) k_emitters(Geo g, Batch b, float4* __restrict__ rad,
                                                  float4* __restrict__ illum, const float* __restrict__ area,
                                                  double tol, DevState* st) {
    if (st->stopped) return;
    __shared__ double red[256];
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
        float4 last = make_float4(0, 0, 0, 0);
        uint32_t nv = 0;
        for (uint32_t h = 0; h < b.K; h++) {
            if (!b.valid[h]) continue;
            nv++;
            const uint32_t e = b.shooters[h];
            float4 r = rad[e], il = illum[e];
            const float4 s = b.saved[h];
            last = r;
            il.x = il.x + s.x; il.y = il.y + s.y; il.z = il.z + s.z;
            r.x = r.x - s.x; r.y = r.y - s.y; r.z = r.z - s.z;
            rad[e] = r;
            illum[e] = il;
        }
        st->shots_done += 1;
        st->hemicubes += (double)nv;
        st->last_energy[0] = last.x;
        st->last_energy[1] = last.y;
        st->last_energy[2] = last.z;
        int stop = 0;
        if (g.mode == 0) stop = (double)sqrtf(last.x * last.x + last.y * last.y + last.z * last.z) < 0.1;
        s_stop = stop;
    }
    __syncthreads();
    int stop = s_stop;
    if (g.mode != 0) {
        const double p = block_unshot_power(rad, area, g.n, red);
        if (threadIdx.x == 0) {
            const double res = st->power0 > 0 ? p / st->power0 : 0.0;
            st->residual = res;
            if (res <= tol) stop = 1;
        }
    }
    if (threadIdx.x == 0 && stop) st->stopped = 1;
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
    k_emitters<<<1, 256, 0, s>>>(g, b, rad, illum, area, tol, st);
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

}  // namespace rad
