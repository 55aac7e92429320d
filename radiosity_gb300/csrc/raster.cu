// Hemicube item-buffer rasteriser and delta-form-factor reduction.
//
// Replaces the reference's OpenGL five-face draw (source/Main.cpp:1155-1198,
// patch-ID shader source/Shaders.cpp:235-260) and the ProcessHemicube OpenCL
// kernel (source/Kernel_ProcessHemicube.h:9-70) with a sort-middle tile
// rasteriser:
//   k_camera   K*5 face MVPs + shooter frame + saved unshot energy
//   k_setup    thread per (hemicube, patch): shooter-plane cull, clip-space
//              transform, trivial frustum/scissor reject, near/far/guard clip,
//              fixed-point snap, back-face cull; emits 64-byte triangle records
//              (warp-aggregated allocation) and counts per-bin references
//   k_scan     exclusive scan of the bin counts
//   k_fill     scatters triangle ids into per-bin lists
//   k_raster   CTA per (hemicube, tile x tile bin): depth|id keys in shared memory
//              (atomicMin = GL_LESS with patch-index draw order), then either the
//              uint32 item buffer or the fused reduction: each pixel's delta FF is
//              an exact multiple of 2^-61, lanes with equal ids are grouped with
//              __match_any_sync, summed exactly with three redux.sync partial sums,
//              and one 64-bit atomicAdd per (warp, id) lands in Fq[hemicube][id].
// The raster rules are spelled out in oracle/oracle.h (the CPU restatement the
// parity tests compare against bit for bit).
#include <cuda_runtime.h>
#include <stdint.h>

#include "camera.cuh"
#include "rad_internal.cuh"

namespace rad {

// ---------------------------------------------------------------------------
// Delta form-factor table (source/FormFactors.cpp:23-67, layout :295-314)
// ---------------------------------------------------------------------------
__global__ void k_fftab(uint32_t W, float* out) {
    const uint32_t H = W, TW = 2 * W, TH = (uint32_t)(H * 1.5), RES = TW * TH;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= RES) return;
    const int n = (int)W;
    const float PI = 3.1415926535897932384626433832795028841931f;
    float hpw = (1.0f / n);
    float pix = (2.0f / n);
    pix *= pix;
    uint32_t x = i % TW, y = i / TW;
    bool front = false;
    uint32_t k;
    if (x >= W / 2 && x < W * 1.5 && y < H) {
        front = true;
        k = y * W + (x - W / 2);
    } else if (x < W / 2 && y < H) {
        k = (H / 2 - x) * W - y - 1;
    } else if (x >= W * 1.5 && y < H) {
        k = (x - (uint32_t)(W * 1.5)) * W + y;
    } else if (x < W && y >= H) {
        k = (y - H) * W + x;
    } else {
        k = ((H / 2 - 1) - (y - H)) * W + (x - W);
    }
    int tx = (int)(k % W), ty = (int)(k / W);
    float v;
    if (front) {
        float dx = ((tx - n / 2) / (n / 2.0f)) + hpw;
        float dy = ((ty - n / 2) / (n / 2.0f)) + hpw;
        float f = (dx * dx + dy * dy + 1);
        f *= f * PI;
        v = pix / f;
    } else {
        float dx = (tx - n / 2) / (n / 2.0f) + hpw;
        float dy = (n / 2 - 1 - ty) / (n / 2.0f) + hpw;
        float f = (dx * dx + dy * dy + 1);
        f *= f * PI;
        v = (pix * (dy + hpw)) / f;
    }
    out[i] = v;
}

void launch_fftab(uint32_t W, float* fftab, cudaStream_t s) {
    uint32_t res = 3 * W * W;
    k_fftab<<<(res + 255) / 256, 256, 0, s>>>(W, fftab);
}

// ---------------------------------------------------------------------------
// Face cameras
// ---------------------------------------------------------------------------
__global__ void k_camera(Geo g, Batch b, const float* __restrict__ verts, const float4* __restrict__ rad,
                         DevState* st) {
    if (st->stopped) return;
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.K * 5) return;
    uint32_t hi = t / 5;
    int face = (int)(t % 5);
    if (!b.valid[hi]) return;
    float q[12];
    const float* src = verts + 12 * (size_t)b.shooters[hi];
#pragma unroll
    for (int i = 0; i < 12; i++) q[i] = src[i];
    float m[16];
    face_mvp(q, face, g.proj, m);
    float* dst = b.mvp + (size_t)t * 16;
#pragma unroll
    for (int i = 0; i < 16; i++) dst[i] = m[i];
    if (face == 0) {
        f3 c, n, u;
        patch_frame(q, c, n, u);
        float* fr = b.frame + (size_t)hi * 8;
        fr[0] = c.x; fr[1] = c.y; fr[2] = c.z;
        fr[3] = n.x; fr[4] = n.y; fr[5] = n.z;
        b.saved[hi] = rad[b.shooters[hi]];
    }
}

void launch_camera(const Geo& g, const Batch& b, const float* verts, const float4* rad, DevState* st,
                   cudaStream_t s) {
    uint32_t n = b.K * 5;
    k_camera<<<(n + 127) / 128, 128, 0, s>>>(g, b, verts, rad, st);
}

// ---------------------------------------------------------------------------
// Triangle setup
// ---------------------------------------------------------------------------
__device__ __forceinline__ float plane_dist(int pl, float4 v) {
    switch (pl) {
        case 0: return v.z + v.w;
        case 1: return v.w - v.z;
        case 2: return kGuard * v.w - v.x;
        case 3: return kGuard * v.w + v.x;
        case 4: return kGuard * v.w - v.y;
        default: return kGuard * v.w + v.y;
    }
}

// Sutherland-Hodgman over near, far and the four guard planes (in that order).
__device__ __noinline__ int clip_polygon(float4* poly, int n) {
    float4 tmp[12];
    float d[12];
    for (int pl = 0; pl < 6 && n > 0; pl++) {
        bool all_in = true;
        for (int i = 0; i < n; i++) {
            d[i] = plane_dist(pl, poly[i]);
            if (!(d[i] >= 0)) all_in = false;
        }
        if (all_in) continue;
        int m = 0;
        for (int i = 0; i < n; i++) {
            int j = (i + 1 == n) ? 0 : i + 1;
            float4 a = poly[i], bb = poly[j];
            bool ain = d[i] >= 0, bin = d[j] >= 0;
            if (ain) tmp[m++] = a;
            if (ain != bin) {
                float t = d[i] / (d[i] - d[j]);
                float4 c;
                c.x = a.x + t * (bb.x - a.x);
                c.y = a.y + t * (bb.y - a.y);
                c.z = a.z + t * (bb.z - a.z);
                c.w = a.w + t * (bb.w - a.w);
                tmp[m++] = c;
            }
        }
        n = m;
        for (int i = 0; i < m; i++) poly[i] = tmp[i];
    }
    return n;
}

__device__ __forceinline__ bool needs_clip(float4 v) {
    return !(v.z + v.w >= 0) || !(v.w - v.z >= 0) || !(kGuard * v.w - v.x >= 0) || !(kGuard * v.w + v.x >= 0) ||
           !(kGuard * v.w - v.y >= 0) || !(kGuard * v.w + v.y >= 0);
}

__device__ __forceinline__ long long floordiv256(long long a) { return (a >= 0) ? a / 256 : -((-a + 255) / 256); }

// Warp-aggregated allocation of n slots; all 32 lanes must call it.
__device__ __forceinline__ uint32_t warp_alloc(uint32_t* counter, uint32_t n) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t x = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    uint32_t total = __shfl_sync(0xffffffffu, x, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + x - n;
}

struct SV {
    int32_t X, Y;
    float D;
};

// Triangle record for (a, b, c); false when culled (area <= 0) or outside the scissor.
__device__ __forceinline__ bool make_tri(SV a, SV b, SV c, uint32_t id, const FaceInfo& F, TriRec& t) {
    long long area2 = ((long long)b.X - a.X) * ((long long)c.Y - a.Y) - ((long long)c.X - a.X) * ((long long)b.Y - a.Y);
    if (area2 <= 0) return false;
    int32_t xmin = min(a.X, min(b.X, c.X)), xmax = max(a.X, max(b.X, c.X));
    int32_t ymin = min(a.Y, min(b.Y, c.Y)), ymax = max(a.Y, max(b.Y, c.Y));
    long long px0 = floordiv256((long long)xmin - 128 + 255), px1 = floordiv256((long long)xmax - 128);
    long long py0 = floordiv256((long long)ymin - 128 + 255), py1 = floordiv256((long long)ymax - 128);
    const int* sc = F.sc;
    if (px0 < sc[0]) px0 = sc[0];
    if (py0 < sc[1]) py0 = sc[1];
    if (px1 > sc[0] + sc[2] - 1) px1 = sc[0] + sc[2] - 1;
    if (py1 > sc[1] + sc[3] - 1) py1 = sc[1] + sc[3] - 1;
    if (px0 > px1 || py0 > py1) return false;
    float fa = (float)area2;
    float e1x = (float)((long long)b.X - a.X), e1y = (float)((long long)b.Y - a.Y);
    float e2x = (float)((long long)c.X - a.X), e2y = (float)((long long)c.Y - a.Y);
    float d1 = b.D - a.D, d2 = c.D - a.D;
    float gx = (d1 * e2y - d2 * e1y) / fa;
    float gy = (d2 * e1x - d1 * e2x) / fa;
    float ox = (float)((long long)sc[0] * 256 + 128 - a.X), oy = (float)((long long)sc[1] * 256 + 128 - a.Y);
    t.X0 = a.X; t.Y0 = a.Y; t.X1 = b.X; t.Y1 = b.Y; t.X2 = c.X; t.Y2 = c.Y;
    t.c0 = (a.D + gx * ox) + gy * oy;
    t.ax = gx * 256.0f;
    t.ay = gy * 256.0f;
    t.id = id;
    t.px0 = (int16_t)px0; t.px1 = (int16_t)px1; t.py0 = (int16_t)py0; t.py1 = (int16_t)py1;
    return true;
}

__device__ __forceinline__ void count_bins(const Geo& g, const Batch& b, uint32_t hi, const FaceInfo& F,
                                           const TriRec& t) {
    const int tile = (int)g.tile;
    int c0 = (t.px0 - F.sc[0]) / tile, c1 = (t.px1 - F.sc[0]) / tile;
    int r0 = (t.py0 - F.sc[1]) / tile, r1 = (t.py1 - F.sc[1]) / tile;
    uint32_t* cnt = b.bin_count + (size_t)hi * g.nb + F.bin_base;
    for (int r = r0; r <= r1; r++)
        for (int c = c0; c <= c1; c++) atomicAdd(&cnt[r * F.bins_x + c], 1u);
}

__global__ void __launch_bounds__(128) k_setup(Geo g, Batch b, const float* __restrict__ verts, DevState* st) {
    if (st->stopped) return;
    const uint32_t hi = blockIdx.y;
    if (!b.valid[hi]) return;
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = p < g.n;
    const float* fr = b.frame + (size_t)hi * 8;
    const float cx = fr[0], cy = fr[1], cz = fr[2], nx = fr[3], ny = fr[4], nz = fr[5];
    float4 cv[4];
    float q[12];
    if (active) {
        const float4* src = reinterpret_cast<const float4*>(verts + 12 * (size_t)p);
        float4 a = __ldg(src), bq = __ldg(src + 1), c = __ldg(src + 2);
        q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w;
        q[4] = bq.x; q[5] = bq.y; q[6] = bq.z; q[7] = bq.w;
        q[8] = c.x; q[9] = c.y; q[10] = c.z; q[11] = c.w;
        bool behind = true;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            float d = ((q[3 * k] - cx) * nx + (q[3 * k + 1] - cy) * ny) + (q[3 * k + 2] - cz) * nz;
            if (!(d < 0)) behind = false;
        }
        if (behind) active = false;
    }
    for (int f = 0; f < 5; f++) {
        const FaceInfo& F = g.face[f];
        bool fa = active;
        if (fa) {
            const float* m = b.mvp + ((size_t)hi * 5 + f) * 16;
            float mm[16];
#pragma unroll
            for (int i = 0; i < 16; i++) mm[i] = __ldg(m + i);
            uint32_t out_any = 0x3F, in_half = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float x = q[3 * k], y = q[3 * k + 1], z = q[3 * k + 2];
                float4 c;
                c.x = ((mm[0] * x + mm[4] * y) + mm[8] * z) + mm[12];
                c.y = ((mm[1] * x + mm[5] * y) + mm[9] * z) + mm[13];
                c.z = ((mm[2] * x + mm[6] * y) + mm[10] * z) + mm[14];
                c.w = ((mm[3] * x + mm[7] * y) + mm[11] * z) + mm[15];
                cv[k] = c;
                uint32_t o = 0;
                if (c.z + c.w < 0) o |= 1;
                if (c.w - c.z < 0) o |= 2;
                if (c.x > c.w) o |= 4;
                if (c.x < -c.w) o |= 8;
                if (c.y > c.w) o |= 16;
                if (c.y < -c.w) o |= 32;
                out_any &= o;
                // scissor half of the side faces (source/Main.cpp:349-389)
                bool keep = true;
                if (f == 0) keep = c.y < 0;        // UP keeps y_ndc < 0
                else if (f == 1) keep = c.y > 0;   // DOWN keeps y_ndc > 0
                else if (f == 2) keep = c.x > 0;   // LEFT keeps x_ndc > 0
                else if (f == 3) keep = c.x < 0;   // RIGHT keeps x_ndc < 0
                if (keep) in_half = 1;
            }
            if (out_any || !in_half) fa = false;
        }
        const float hw = 0.5f * (float)F.vp[2], hh = 0.5f * (float)F.vp[3];
        const float vx = (float)F.vp[0], vy = (float)F.vp[1];
        for (int t = 0; t < 2; t++) {
            float4 poly[12];
            int pn = 0;
            if (fa) {
                poly[0] = cv[0];
                poly[1] = cv[t == 0 ? 1 : 2];
                poly[2] = cv[t == 0 ? 2 : 3];
                pn = 3;
                if (needs_clip(poly[0]) || needs_clip(poly[1]) || needs_clip(poly[2])) pn = clip_polygon(poly, 3);
            }
            SV sv[12];
            if (pn >= 3) {
                for (int k = 0; k < pn; k++) {
                    float4 c = poly[k];
                    if (!(c.w > 0)) {
                        pn = 0;
                        break;
                    }
                    float xd = c.x / c.w, yd = c.y / c.w;
                    float xw = (xd + 1.0f) * hw + vx, yw = (yd + 1.0f) * hh + vy;
                    sv[k].X = (int32_t)__float2ll_rn(xw * 256.0f);
                    sv[k].Y = (int32_t)__float2ll_rn(yw * 256.0f);
                    sv[k].D = 1.0f / c.w;
                }
            }
            uint32_t ncand = pn >= 3 ? (uint32_t)(pn - 2) : 0u;
            uint32_t base = warp_alloc(&st->tri_count, ncand);
            for (uint32_t j = 0; j < ncand; j++) {
                uint32_t slot = base + j;
                if (slot >= b.tri_cap) {
                    atomicOr(&st->overflow, 1u);
                    break;
                }
                TriRec rec;
                bool ok = make_tri(sv[0], sv[j + 1], sv[j + 2], p, F, rec);
                if (ok) {
                    rec.hf = hi * 5 + (uint32_t)f;
                    b.tris[slot] = rec;
                    count_bins(g, b, hi, F, rec);
                } else {
                    b.tris[slot].id = kDeadTri;
                }
            }
        }
    }
}

void launch_setup(const Geo& g, const Batch& b, const float* verts, DevState* st, cudaStream_t s) {
    dim3 grid((g.n + 127) / 128, b.K);
    k_setup<<<grid, 128, 0, s>>>(g, b, verts, st);
}

// ---------------------------------------------------------------------------
// Bin lists
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_scan(Geo g, Batch b, DevState* st) {
    if (st->stopped) return;
    const uint32_t total = b.K * g.nb;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t per = (total + nt - 1) / nt;
    const uint32_t lo = tid * per, hi = min(total, lo + per);
    uint32_t s = 0;
    for (uint32_t i = lo; i < hi; i++) s += b.bin_count[i];
    __shared__ uint32_t part[1024];
    part[tid] = s;
    __syncthreads();
    for (uint32_t o = 1; o < nt; o <<= 1) {
        uint32_t v = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    uint32_t run = part[tid] - s;
    for (uint32_t i = lo; i < hi; i++) {
        b.bin_offset[i] = run;
        b.bin_fill[i] = 0;
        run += b.bin_count[i];
    }
    if (tid == nt - 1 && part[tid] > b.list_cap) atomicOr(&st->overflow, 2u);
}

__global__ void k_fill(Geo g, Batch b, DevState* st) {
    if (st->stopped) return;
    const uint32_t ntri = min(st->tri_count, b.tri_cap);
    const int tile = (int)g.tile;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ntri; s += gridDim.x * blockDim.x) {
        const TriRec& t = b.tris[s];
        if (t.id == kDeadTri) continue;
        uint32_t hi = t.hf / 5, f = t.hf % 5;
        const FaceInfo& F = g.face[f];
        int c0 = (t.px0 - F.sc[0]) / tile, c1 = (t.px1 - F.sc[0]) / tile;
        int r0 = (t.py0 - F.sc[1]) / tile, r1 = (t.py1 - F.sc[1]) / tile;
        size_t gb0 = (size_t)hi * g.nb + F.bin_base;
        for (int r = r0; r <= r1; r++)
            for (int c = c0; c <= c1; c++) {
                size_t gb = gb0 + r * F.bins_x + c;
                uint32_t pos = atomicAdd(&b.bin_fill[gb], 1u);
                uint32_t idx = b.bin_offset[gb] + pos;
                if (idx < b.list_cap) b.bin_list[idx] = s;
            }
    }
}

void launch_bins(const Geo& g, const Batch& b, DevState* st, cudaStream_t s) {
    k_scan<<<1, 1024, 0, s>>>(g, b, st);
    k_fill<<<152 * 8, 256, 0, s>>>(g, b, st);
}

// ---------------------------------------------------------------------------
// Raster + reduction
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t depth_ordinal(float d) {
    if (!(d > 0)) return 0x7F800000u;
    uint32_t bits = __float_as_uint(d);
    if (bits >= 0x7F800000u) return 0;
    return 0x7F800000u - bits;
}

// Exact warp-segmented sum of q over lanes sharing `key`; returns the group's sum
// on every lane and the group mask in *gm.
__device__ __forceinline__ unsigned long long group_sum(uint32_t key, unsigned long long q, unsigned* gm) {
    unsigned m = __match_any_sync(0xffffffffu, key);
    uint32_t a = (uint32_t)(q & 0x1FFFFFull), bb = (uint32_t)((q >> 21) & 0x1FFFFFull), c = (uint32_t)(q >> 42);
    uint32_t sa = __reduce_add_sync(m, a), sb = __reduce_add_sync(m, bb), sc = __reduce_add_sync(m, c);
    *gm = m;
    return (unsigned long long)sa + ((unsigned long long)sb << 21) + ((unsigned long long)sc << 42);
}

template <int TILE>
__global__ void __launch_bounds__(256) k_raster(Geo g, Batch b, const float* __restrict__ fftab, DevState* st,
                                                int write_items, int fused) {
    if (st->stopped) return;
    const uint32_t gb = blockIdx.x;
    const uint32_t hi = gb / g.nb, bin = gb % g.nb;
    const BinInfo bi = b.bins[bin];
    const bool valid = b.valid[hi] != 0;
    __shared__ unsigned long long key[TILE * TILE];
    for (int j = threadIdx.x; j < TILE * TILE; j += blockDim.x) key[j] = ~0ull;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    if (valid) {
        const FaceInfo& F = g.face[bi.face];
        const int sx = F.sc[0], sy = F.sc[1];
        uint32_t cnt = b.bin_count[gb], off = b.bin_offset[gb];
        if (off >= b.list_cap) cnt = 0;
        else if (off + cnt > b.list_cap) cnt = b.list_cap - off;
        const int bx1 = bi.x0 + bi.w - 1, by1 = bi.y0 + bi.h - 1;
        for (uint32_t i = warp; i < cnt; i += nwarp) {
            const TriRec t = b.tris[b.bin_list[off + i]];
            const int x0 = max((int)t.px0, (int)bi.x0), x1 = min((int)t.px1, bx1);
            const int y0 = max((int)t.py0, (int)bi.y0), y1 = min((int)t.py1, by1);
            if (x0 > x1 || y0 > y1) continue;
            const long long dx0 = (long long)t.X1 - t.X0, dy0 = (long long)t.Y1 - t.Y0;
            const long long dx1 = (long long)t.X2 - t.X1, dy1 = (long long)t.Y2 - t.Y1;
            const long long dx2 = (long long)t.X0 - t.X2, dy2 = (long long)t.Y0 - t.Y2;
            const bool tl0 = (t.Y1 < t.Y0) || (t.Y1 == t.Y0 && t.X1 < t.X0);
            const bool tl1 = (t.Y2 < t.Y1) || (t.Y2 == t.Y1 && t.X2 < t.X1);
            const bool tl2 = (t.Y0 < t.Y2) || (t.Y0 == t.Y2 && t.X0 < t.X2);
            const int nsx = (x1 - x0 + 8) >> 3, nsy = (y1 - y0 + 4) >> 2;
            for (int s = 0; s < nsx * nsy; s++) {
                const int px = x0 + (s % nsx) * 8 + (lane & 7);
                const int py = y0 + (s / nsx) * 4 + (lane >> 3);
                if (px > x1 || py > y1) continue;
                const long long PX = (long long)px * 256 + 128, PY = (long long)py * 256 + 128;
                const long long e0 = dx0 * (PY - t.Y0) - dy0 * (PX - t.X0);
                const long long e1 = dx1 * (PY - t.Y1) - dy1 * (PX - t.X1);
                const long long e2 = dx2 * (PY - t.Y2) - dy2 * (PX - t.X2);
                const bool in = (e0 > 0 || (e0 == 0 && tl0)) && (e1 > 0 || (e1 == 0 && tl1)) &&
                                (e2 > 0 || (e2 == 0 && tl2));
                if (!in) continue;
                const float u = (float)(px - sx), w = (float)(py - sy);
                const float D = (t.c0 + t.ax * u) + t.ay * w;
                const unsigned long long k = ((unsigned long long)depth_ordinal(D) << 32) | t.id;
                atomicMin(&key[(py - bi.y0) * TILE + (px - bi.x0)], k);
            }
        }
    }
    __syncthreads();
    const size_t img = (size_t)hi * g.RES;
    for (int j = threadIdx.x; j < TILE * TILE; j += blockDim.x) {
        const int ly = j / TILE, lx = j % TILE;
        const bool inb = lx < bi.w && ly < bi.h;
        const int px = bi.x0 + lx, py = bi.y0 + ly;
        const unsigned long long k = key[j];
        const bool has = inb && valid && k != ~0ull;
        const uint32_t id = has ? (uint32_t)(k & 0xFFFFFFFFull) : 0xFFFFFFFFu;
        if (write_items && inb) b.items[img + (size_t)py * g.TW + px] = has ? id + 1 : 0u;
        if (fused) {
            unsigned long long q = 0;
            if (has) q = __float2ull_rz(fftab[(size_t)py * g.TW + px] * 0x1p61f);
            unsigned gm;
            unsigned long long sum = group_sum(id, q, &gm);
            if (has && lane == __ffs(gm) - 1) atomicAdd(&b.Fq[(size_t)hi * g.n + id], sum);
        }
    }
}

void launch_raster(const Geo& g, const Batch& b, const float* fftab, DevState* st, bool write_items,
                   bool fused_reduce, cudaStream_t s) {
    dim3 grid(b.K * g.nb);
    switch (g.tile) {
        case 16: k_raster<16><<<grid, 256, 0, s>>>(g, b, fftab, st, write_items, fused_reduce); break;
        case 64: k_raster<64><<<grid, 256, 0, s>>>(g, b, fftab, st, write_items, fused_reduce); break;
        default: k_raster<32><<<grid, 256, 0, s>>>(g, b, fftab, st, write_items, fused_reduce); break;
    }
}

// Reduction of caller-provided item buffers (count stacked 2W x 1.5W images).
__global__ void k_reduce_items(Geo g, Batch b, const float* __restrict__ fftab, uint32_t count) {
    const size_t total = (size_t)count * g.RES;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t it = idx < total ? b.items[idx] : 0u;
    const bool has = it != 0 && it <= g.n;
    const uint32_t hi = (uint32_t)(idx / g.RES), pix = (uint32_t)(idx % g.RES);
    unsigned long long q = 0;
    if (has) q = __float2ull_rz(fftab[pix] * 0x1p61f);
    // lanes of one warp may straddle two images: fold the image into the key
    const uint32_t key = has ? (it - 1) ^ (hi << 31) : 0xFFFFFFFFu;
    unsigned gm;
    unsigned long long sum = group_sum(has ? key : 0xFFFFFFFFu, q, &gm);
    if (has && lane == __ffs(gm) - 1) atomicAdd(&b.Fq[(size_t)hi * g.n + (it - 1)], sum);
}

void launch_reduce_items(const Geo& g, const Batch& b, const float* fftab, uint32_t count, cudaStream_t s) {
    size_t total = (size_t)count * g.RES;
    k_reduce_items<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(g, b, fftab, count);
}

__global__ void k_fq_to_float(const unsigned long long* __restrict__ Fq, size_t total, float* out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __ull2float_rn(Fq[i]) * 0x1p-61f;
}

void launch_fq_to_float(const Geo& g, const Batch& b, uint32_t count, float* out, cudaStream_t s) {
    size_t total = (size_t)count * g.n;
    k_fq_to_float<<<152 * 4, 256, 0, s>>>(b.Fq, total, out);
}

}  // namespace rad
