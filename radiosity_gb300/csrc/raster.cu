// Hemicube item-buffer rasteriser and delta-form-factor reduction.
//
// Replaces the reference's OpenGL five-face draw (source/Main.cpp:1155-1198,
// patch-ID shader source/Shaders.cpp:235-260) and the ProcessHemicube OpenCL
// kernel (source/Kernel_ProcessHemicube.h:9-70) with a sort-middle tile
// rasteriser:
//   k_camera   K*5 face MVPs + shooter frame + saved unshot energy
//   k_setup    thread per (hemicube, patch): shooter-plane cull, exact per-face
//              mask, clip-space transform, near/far/guard clip, fixed-point snap,
//              back-face cull; emits one 64-byte record per patch quad and face
//              (both triangles; warp-aggregated allocation) and counts per-bin
//              references
//   k_scan     exclusive scan of the bin counts
//   k_fill     scatters record indices into per-bin lists
//   k_raster   CTA per (hemicube, tile x tile bin): depth|id keys in shared memory
//              (atomicMin = GL_LESS with patch-index draw order).  Small records
//              (extent <= 64 px) are rasterised by exact integer row spans laid out as
//              one packed pixel stream per warp; big triangles one warp each in 8x4
//              stamps.  Then either the uint32 item buffer or the fused reduction:
//              each pixel's delta FF is an exact multiple of 2^-61, summed per run of
//              equal ids down each column and added to Fq[hemicube][id] with one 64-bit
//              atomic per run.  k_reduce_items does the same for caller item buffers
//              with __match_any_sync groups and exact redux.sync sums.
// The raster rules are spelled out in oracle/oracle.h (the CPU restatement the
// parity tests compare against bit for bit).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

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

// Cull test of (a, b, c): CCW with positive area and a non-empty pixel bbox inside
// the scissor; the bbox is returned in px (x0, x1, y0, y1).
__device__ __forceinline__ bool tri_bbox(SV a, SV b, SV c, const FaceInfo& F, int* px) {
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
    px[0] = (int)px0; px[1] = (int)px1; px[2] = (int)py0; px[3] = (int)py1;
    return true;
}

// Depth-plane gradients x256 of a triangle that passed tri_bbox (the float operations
// of the oracle's plane set-up, in the same order).
__device__ __forceinline__ void tri_plane(SV a, SV b, SV c, float* ax, float* ay) {
    const long long area2 =
        ((long long)b.X - a.X) * ((long long)c.Y - a.Y) - ((long long)c.X - a.X) * ((long long)b.Y - a.Y);
    // correctly rounded either way; the 32-bit conversion serves the usual small triangle
    float fa = (area2 >= INT32_MIN && area2 <= INT32_MAX) ? (float)(int32_t)area2 : (float)area2;
    // the coordinate differences fit in 32 bits (|X|, |Y| < 2^28 for W <= 2048): 32-bit
    // conversions of the same integers, off the slow 64-bit conversion path
    float e1x = (float)(b.X - a.X), e1y = (float)(b.Y - a.Y);
    float e2x = (float)(c.X - a.X), e2y = (float)(c.Y - a.Y);
    float d1 = b.D - a.D, d2 = c.D - a.D;
    float gx = (d1 * e2y - d2 * e1y) / fa;
    float gy = (d2 * e1x - d1 * e2x) / fa;
    *ax = gx * 256.0f;  // exact: a power-of-two scale of a value far from overflow
    *ay = gy * 256.0f;
}

// Writes the record of triangles A = (v0,v1,v2) (when okA, box pa) and B = (v0,v2,v3)
// (when okB, box pb); at least one is set.  The record's box is the union of the two.
__device__ __forceinline__ void rec_write(const SV* v, bool okA, bool okB, const int* pa, const int* pb, uint32_t id,
                                          int face, TriRec* out) {
    float axA = 0.f, ayA = 0.f, axB = 0.f, ayB = 0.f;
    int bx0, bx1, by0, by1;
    if (okA) {
        tri_plane(v[0], v[1], v[2], &axA, &ayA);
        bx0 = pa[0]; bx1 = pa[1]; by0 = pa[2]; by1 = pa[3];
        if (okB) {
            bx0 = min(bx0, pb[0]); bx1 = max(bx1, pb[1]); by0 = min(by0, pb[2]); by1 = max(by1, pb[3]);
        }
    } else {
        bx0 = pb[0]; bx1 = pb[1]; by0 = pb[2]; by1 = pb[3];
    }
    if (okB) tri_plane(v[0], v[2], v[3], &axB, &ayB);
    const uint32_t bx = (uint32_t)bx0 | ((uint32_t)bx1 << 12) | ((uint32_t)face << 24) | (okA ? kRecA : 0u) |
                        (okB ? kRecB : 0u);
    const uint32_t by = (uint32_t)by0 | ((uint32_t)by1 << 12);
    int4* o = reinterpret_cast<int4*>(out);
    o[0] = make_int4(v[0].X, v[1].X, v[2].X, v[3].X);
    o[1] = make_int4(v[0].Y, v[1].Y, v[2].Y, v[3].Y);
    o[2] = make_int4(__float_as_int(v[0].D), __float_as_int(axA), __float_as_int(axB), __float_as_int(ayA));
    o[3] = make_int4(__float_as_int(ayB), (int)id, (int)bx, (int)by);
}

// Union of two clamped boxes (x0, x1, y0, y1) where either may be absent.
__device__ __forceinline__ void box_union(bool okA, bool okB, const int* pa, const int* pb, int* out) {
    if (okA && okB) {
        out[0] = min(pa[0], pb[0]); out[1] = max(pa[1], pb[1]);
        out[2] = min(pa[2], pb[2]); out[3] = max(pa[3], pb[3]);
    } else {
        const int* p = okA ? pa : pb;
        out[0] = p[0]; out[1] = p[1]; out[2] = p[2]; out[3] = p[3];
    }
}

// Adds one to each bin the pixel box px touches; cnt = the hemicube's global bin counters.
__device__ __forceinline__ void count_bins(const Geo& g, const FaceInfo& F, const int* px, uint32_t* cnt) {
    const int sh = (int)g.tile_shift;  // boxes lie inside the scissor: offsets are >= 0
    const int c0 = (px[0] - F.sc[0]) >> sh, c1 = (px[1] - F.sc[0]) >> sh;
    const int r0 = (px[2] - F.sc[1]) >> sh, r1 = (px[3] - F.sc[1]) >> sh;
    cnt += F.bin_base;
    for (int r = r0; r <= r1; r++)
        for (int c = c0; c <= c1; c++) atomicAdd(&cnt[r * F.bins_x + c], 1u);
}

// count_bins for the fast path, called by all 32 lanes: triangles that touch a
// single bin (most of them) are grouped by bin with __match_any_sync and counted
// with one atomic per group; the others count their bins one by one.
__device__ __forceinline__ void count_bins_warp(const Geo& g, const Batch& b, uint32_t hi, const FaceInfo& F,
                                                const int* px, bool on) {
    const int sh = (int)g.tile_shift;
    int c0 = 0, c1 = -1, r0 = 0, r1 = -1;
    if (on) {
        c0 = (px[0] - F.sc[0]) >> sh;
        c1 = (px[1] - F.sc[0]) >> sh;
        r0 = (px[2] - F.sc[1]) >> sh;
        r1 = (px[3] - F.sc[1]) >> sh;
    }
    uint32_t* cnt = b.bin_count + (size_t)hi * g.nb;
    const bool single = on && c0 == c1 && r0 == r1;
    // the hemicube-wide bin index: the lanes of a warp may draw different faces
    const uint32_t key = single ? (uint32_t)(F.bin_base + r0 * F.bins_x + c0) : 0xFFFFFFFFu;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    if (single && (threadIdx.x & 31) == (unsigned)(__ffs(grp) - 1)) atomicAdd(&cnt[key], (uint32_t)__popc(grp));
    if (on && !single)
        for (int r = r0; r <= r1; r++)
            for (int c = c0; c <= c1; c++) atomicAdd(&cnt[F.bin_base + r * F.bins_x + c], 1u);
}

// Snap one clip-space vertex to 24.8 fixed-point window coordinates; false when w <= 0.
__device__ __forceinline__ bool snap_vertex(float4 c, float hw, float hh, float vx, float vy, SV& o) {
    if (!(c.w > 0)) return false;
    const float xd = c.x / c.w, yd = c.y / c.w;
    const float xw = (xd + 1.0f) * hw + vx, yw = (yd + 1.0f) * hh + vy;
    // inside the guard band |xw * 256| < 2^28 (W <= 2048): a 32-bit round-to-nearest-even
    // conversion, the same value as the 64-bit one
    o.X = __float2int_rn(xw * 256.0f);
    o.Y = __float2int_rn(yw * 256.0f);
    o.D = 1.0f / c.w;
    return true;
}

// Records of a clipped polygon's fan (s0, sj, sj+1), two triangles per record, into slots
// base .. base + (pn-1)/2 - 1; a record whose triangles are both culled is marked dead.
__device__ __forceinline__ uint32_t fan_records(int pn) { return pn >= 3 ? (uint32_t)(pn - 1) / 2u : 0u; }

__device__ __noinline__ void emit_polygon(const Geo& g, const Batch& b, const float4* poly, int pn, uint32_t base,
                                          uint32_t p, uint32_t hi, int f, float hw, float hh, float vx, float vy,
                                          uint32_t* cnt, DevState* st) {
    const FaceInfo& F = g.face[f];
    SV sv[12];
    bool good = true;
    for (int k = 0; k < pn; k++) good = good && snap_vertex(poly[k], hw, hh, vx, vy, sv[k]);
    TriRec* tris = b.tris + (size_t)hi * b.tri_cap_h;  // this hemicube's records
    for (int j = 1, r = 0; j + 1 < pn; j += 2, r++) {
        const uint32_t slot = base + (uint32_t)r;
        if (slot >= b.tri_cap_h) {
            atomicOr(&st->overflow, 1u);
            return;
        }
        const bool hasB = j + 2 < pn;
        SV v[4] = {sv[0], sv[j], sv[j + 1], hasB ? sv[j + 2] : sv[j + 1]};
        int pa[4], pb[4], px[4];
        const bool okA = good && tri_bbox(v[0], v[1], v[2], F, pa);
        const bool okB = good && hasB && tri_bbox(v[0], v[2], v[3], F, pb);
        if (okA || okB) {
            rec_write(v, okA, okB, pa, pb, p, f, &tris[slot]);
            box_union(okA, okB, pa, pb, px);
            count_bins(g, F, px, cnt);
        } else {
            tris[slot].id = kDeadTri;
        }
    }
}

// Clip-space corners of quad q (12 floats) under face f's MVP mm, and whether the quad
// can cover a pixel of face f: not all corners outside one clip plane, and at least one
// corner on the kept half of a side face (source/Main.cpp:349-389).
__device__ __forceinline__ bool face_corners(const float* q, const float* mm, int f, float4* cv) {
    uint32_t out_any = 0x3F, in_half = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float x = q[3 * k], y = q[3 * k + 1], z = q[3 * k + 2];
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
        bool keep = true;
        if (f == 0) keep = c.y < 0;        // UP keeps y_ndc < 0
        else if (f == 1) keep = c.y > 0;   // DOWN keeps y_ndc > 0
        else if (f == 2) keep = c.x > 0;   // LEFT keeps x_ndc > 0
        else if (f == 3) keep = c.x < 0;   // RIGHT keeps x_ndc < 0
        if (keep) in_half = 1;
    }
    return !out_any && in_half;
}

__device__ __forceinline__ void load_quad(const float* verts, uint32_t p, float* q) {
    const float4* src = reinterpret_cast<const float4*>(verts + 12 * (size_t)p);
    const float4 a = __ldg(src), bq = __ldg(src + 1), c = __ldg(src + 2);
    q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w;
    q[4] = bq.x; q[5] = bq.y; q[6] = bq.z; q[7] = bq.w;
    q[8] = c.x; q[9] = c.y; q[10] = c.z; q[11] = c.w;
}

// Bounding box (min xyz, max xyz) of each group of 128 consecutive patches: the patches of one
// k_setup CTA.  One CTA per group.
__global__ void __launch_bounds__(128) k_group_boxes(const float* __restrict__ verts, uint32_t n, float* gbox) {
    __shared__ float s_lo[3][4], s_hi[3][4];
    const uint32_t p = blockIdx.x * 128 + threadIdx.x;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (p < n)
        for (int k = 0; k < 4; k++)
            for (int d = 0; d < 3; d++) {
                const float v = verts[12 * (size_t)p + 3 * k + d];
                lo[d] = fminf(lo[d], v);
                hi[d] = fmaxf(hi[d], v);
            }
    for (int d = 0; d < 3; d++)
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; d++) {
            s_lo[d][threadIdx.x >> 5] = lo[d];
            s_hi[d][threadIdx.x >> 5] = hi[d];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        gbox[6 * blockIdx.x + d] = fminf(fminf(s_lo[d][0], s_lo[d][1]), fminf(s_lo[d][2], s_lo[d][3]));
        gbox[6 * blockIdx.x + 3 + d] = fmaxf(fmaxf(s_hi[d][0], s_hi[d][1]), fmaxf(s_hi[d][2], s_hi[d][3]));
    }
}

void launch_group_boxes(const float* verts, uint32_t n, float* gbox, cudaStream_t s) {
    k_group_boxes<<<(n + 127) / 128, 128, 0, s>>>(verts, n, gbox);
}

// Which faces the CTA's group box may touch, and whether any of it lies in front of the
// shooter's tangent plane.  48 threads, one per (task, box corner): tasks 0-4 are the faces,
// task 5 the tangent plane.  A face is impossible when all 8 corners lie outside one clip
// plane, or (side faces) all outside the kept half, and the group is behind when all 8
// corners are behind the plane; each test keeps a margin of 1e-5 of the largest sum of
// absolute terms, far above the rounding of the per-patch tests, which use the same
// expressions on points inside the box.  Bit 5 of the result: some corner is not behind.
__device__ __forceinline__ uint32_t group_face_mask(const float* __restrict__ box, const float* s_mvp,
                                                    const float* s_fr) {
    const uint32_t t = threadIdx.x, task = t >> 3, k = t & 7;
    const float x = box[(k & 1) ? 3 : 0], y = box[(k & 2) ? 4 : 1], z = box[(k & 4) ? 5 : 2];
    constexpr float kEps = 1e-5f;
    float u[7], m[7];  // value (inside when >= 0) and magnitude per test
#pragma unroll
    for (int j = 0; j < 7; j++) u[j] = m[j] = 0.f;
    if (task < 5) {
        const float* mm = s_mvp + task * 16;
        const float cx = ((mm[0] * x + mm[4] * y) + mm[8] * z) + mm[12];
        const float cy = ((mm[1] * x + mm[5] * y) + mm[9] * z) + mm[13];
        const float cz = ((mm[2] * x + mm[6] * y) + mm[10] * z) + mm[14];
        const float cw = ((mm[3] * x + mm[7] * y) + mm[11] * z) + mm[15];
        const float ax = ((fabsf(mm[0] * x) + fabsf(mm[4] * y)) + fabsf(mm[8] * z)) + fabsf(mm[12]);
        const float ay = ((fabsf(mm[1] * x) + fabsf(mm[5] * y)) + fabsf(mm[9] * z)) + fabsf(mm[13]);
        const float az = ((fabsf(mm[2] * x) + fabsf(mm[6] * y)) + fabsf(mm[10] * z)) + fabsf(mm[14]);
        const float aw = ((fabsf(mm[3] * x) + fabsf(mm[7] * y)) + fabsf(mm[11] * z)) + fabsf(mm[15]);
        u[0] = cz + cw; m[0] = az + aw;  // near
        u[1] = cw - cz; m[1] = az + aw;  // far
        u[2] = cw - cx; m[2] = ax + aw;  // x <= w
        u[3] = cw + cx; m[3] = ax + aw;  // x >= -w
        u[4] = cw - cy; m[4] = ay + aw;  // y <= w
        u[5] = cw + cy; m[5] = ay + aw;  // y >= -w
        // the kept half of a side face (inside when > 0); the front face keeps everything
        u[6] = task == 0 ? -cy : (task == 1 ? cy : (task == 2 ? cx : (task == 3 ? -cx : 1.f)));
        m[6] = task <= 1 ? ay : (task <= 3 ? ax : 0.f);
    } else if (task == 5) {
        const float dx = x - s_fr[0], dy = y - s_fr[1], dz = z - s_fr[2];
        u[0] = (dx * s_fr[3] + dy * s_fr[4]) + dz * s_fr[5];  // in front when >= 0
        m[0] = (fabsf(dx * s_fr[3]) + fabsf(dy * s_fr[4])) + fabsf(dz * s_fr[5]);
    }
    // max over the 8 corners (lanes of one 8-lane group)
#pragma unroll
    for (int j = 0; j < 7; j++)
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            u[j] = fmaxf(u[j], __shfl_xor_sync(0xffffffffu, u[j], o));
            m[j] = fmaxf(m[j], __shfl_xor_sync(0xffffffffu, m[j], o));
        }
    bool possible;
    if (task < 5) {
        possible = true;
#pragma unroll
        for (int j = 0; j < 6; j++)
            if (u[j] < -kEps * m[j]) possible = false;  // every corner outside plane j
        if (u[6] <= -kEps * m[6] && task < 4) possible = false;  // every corner outside the half
    } else {
        possible = !(u[0] < -kEps * m[0]);  // not every corner behind
    }
    return possible ? 1u << task : 0u;
}

// Thread per (hemicube, patch) in three phases, after a per-CTA test of the group's bounding
// box (group_face_mask) that skips faces no patch of the group can touch and the whole CTA when
// the group lies behind the shooter:
//  1. tangent-plane cull and the exact per-face test -> a 5-bit mask of faces to draw;
//  2. warp compaction of the (patch, face) items;
//  3. the warp's items, one per lane with all lanes busy: corners again, clip or snap,
//     records, bin counts.
__global__ void __launch_bounds__(128, 8) k_setup(Geo g, Batch b, const float* __restrict__ verts,
                                                  const float* __restrict__ gbox, DevState* st) {
    if (st->stopped) return;
    const uint32_t hi = blockIdx.y;
    if (!b.valid[hi]) return;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ float s_mvp[5 * 16];
    __shared__ float s_fr[8];
    __shared__ uint8_t s_items[4][32 * 5];  // (lane << 3) | face
    __shared__ uint32_t s_clipq[4][32 * 5]; // per warp: items that need clipping, (patch << 3) | face
    __shared__ uint32_t s_nclip[4];
    // bin counts go straight to the hemicube's global counters (warp-aggregated for the
    // records that touch one bin): no shared histogram, so no barrier before its flush
    uint32_t* cnt = b.bin_count + (size_t)hi * g.nb;
    for (int i = threadIdx.x; i < 5 * 16; i += blockDim.x) s_mvp[i] = b.mvp[(size_t)hi * 80 + i];
    if (threadIdx.x < 8) s_fr[threadIdx.x] = b.frame[(size_t)hi * 8 + threadIdx.x];
    __shared__ uint32_t s_gmask;
    if (lane == 0) s_nclip[warp] = 0;
    if (threadIdx.x == 0) s_gmask = 0;
    __syncthreads();
    if (threadIdx.x < 64) {  // warps 0 and 1: the group's face mask (48 of their lanes)
        const uint32_t bit = group_face_mask(gbox + 6 * (size_t)blockIdx.x, s_mvp, s_fr);
        if (bit && threadIdx.x < 48 && (threadIdx.x & 7) == 0) atomicOr(&s_gmask, bit);
    }
    __syncthreads();
    const uint32_t gmask = s_gmask;
    if (!(gmask & 32u)) return;  // the whole group is behind the shooter
    // 1. cull + face mask
    uint32_t mask = 0;
    if (p < g.n) {
        const float cx = s_fr[0], cy = s_fr[1], cz = s_fr[2], nx = s_fr[3], ny = s_fr[4], nz = s_fr[5];
        float q[12];
        load_quad(verts, p, q);
        bool behind = true;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float d = ((q[3 * k] - cx) * nx + (q[3 * k + 1] - cy) * ny) + (q[3 * k + 2] - cz) * nz;
            if (!(d < 0)) behind = false;
        }
        if (!behind)
            for (int f = 0; f < 5; f++) {
                if (!((gmask >> f) & 1u)) continue;  // no patch of the group can touch face f
                // the z and w rows first: all four corners outside the near plane
                // (z + w < 0) reject the face without the x and y rows.  The rows are the
                // same float expressions as face_corners', and the tests below are its
                // tests on the same values, so the mask is unchanged.
                const float* mm = s_mvp + f * 16;
                float cz[4], cw[4];
                bool near_out = true;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float x = q[3 * k], y = q[3 * k + 1], z = q[3 * k + 2];
                    cz[k] = ((mm[2] * x + mm[6] * y) + mm[10] * z) + mm[14];
                    cw[k] = ((mm[3] * x + mm[7] * y) + mm[11] * z) + mm[15];
                    if (!(cz[k] + cw[k] < 0)) near_out = false;
                }
                if (near_out) continue;
                uint32_t out_any = 0x3F, in_half = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float x = q[3 * k], y = q[3 * k + 1], z = q[3 * k + 2];
                    const float cx = ((mm[0] * x + mm[4] * y) + mm[8] * z) + mm[12];
                    const float cy = ((mm[1] * x + mm[5] * y) + mm[9] * z) + mm[13];
                    uint32_t o = 0;
                    if (cz[k] + cw[k] < 0) o |= 1;
                    if (cw[k] - cz[k] < 0) o |= 2;
                    if (cx > cw[k]) o |= 4;
                    if (cx < -cw[k]) o |= 8;
                    if (cy > cw[k]) o |= 16;
                    if (cy < -cw[k]) o |= 32;
                    out_any &= o;
                    const bool keep = f == 0 ? cy < 0 : (f == 1 ? cy > 0 : (f == 2 ? cx > 0 : (f == 3 ? cx < 0 : true)));
                    if (keep) in_half = 1;
                }
                if (!out_any && in_half) mask |= 1u << f;
            }
    }
    // 2. compaction
    const uint32_t nmine = __popc(mask);
    uint32_t incl = nmine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint8_t* items = s_items[warp];
    {
        uint32_t k = incl - nmine;
        for (int f = 0; f < 5; f++)
            if ((mask >> f) & 1u) items[k++] = (uint8_t)((lane << 3) | (uint32_t)f);
    }
    __syncwarp();
    // 3. items, 32 at a time.  An item whose four corners need no clipping is one record
    //    (both triangles).  Items that need clipping (a few percent, but enough to put
    //    one in about half of all 32-item groups) are queued and clipped afterwards in
    //    compact groups, so the common path does not wait for them.
    const uint32_t pbase = blockIdx.x * blockDim.x + warp * 32;
    for (uint32_t r = 0; r < total; r += 32) {
        const bool has = r + lane < total;
        uint32_t pp = 0;
        int f = 0;
        if (has) {
            const uint32_t it = items[r + lane];
            pp = pbase + (it >> 3);
            f = (int)(it & 7u);
        }
        const FaceInfo& F = g.face[f];
        float4 cv[4];
        if (has) {
            float q[12];
            load_quad(verts, pp, q);
            face_corners(q, s_mvp + f * 16, f, cv);
        }
        const bool clipq =
            has && (needs_clip(cv[0]) || needs_clip(cv[1]) || needs_clip(cv[2]) || needs_clip(cv[3]));
        const uint32_t qpos = warp_alloc(&s_nclip[warp], clipq ? 1u : 0u);
        if (clipq) s_clipq[warp][qpos] = (pp << 3) | (uint32_t)f;
        SV sv[4];
        int pa[4], pb[4], px[4];
        bool okA = false, okB = false;
        if (has && !clipq) {
            const float hw = 0.5f * (float)F.vp[2], hh = 0.5f * (float)F.vp[3];
            const float vx = (float)F.vp[0], vy = (float)F.vp[1];
            const bool g0 = snap_vertex(cv[0], hw, hh, vx, vy, sv[0]), g1 = snap_vertex(cv[1], hw, hh, vx, vy, sv[1]);
            const bool g2 = snap_vertex(cv[2], hw, hh, vx, vy, sv[2]), g3 = snap_vertex(cv[3], hw, hh, vx, vy, sv[3]);
            okA = g0 && g1 && g2 && tri_bbox(sv[0], sv[1], sv[2], F, pa);
            okB = g0 && g2 && g3 && tri_bbox(sv[0], sv[2], sv[3], F, pb);
        }
        const bool quad = okA || okB;
        // slots are allocated per hemicube (one counter each, not one for the batch)
        const uint32_t base = warp_alloc(&b.tri_counts[hi], quad ? 1u : 0u);
        const bool written = quad && base < b.tri_cap_h;
        if (quad) {
            if (!written) atomicOr(&st->overflow, 1u);
            else rec_write(sv, okA, okB, pa, pb, pp, f, &b.tris[(size_t)hi * b.tri_cap_h + base]);
            box_union(okA, okB, pa, pb, px);
        }
        count_bins_warp(g, b, hi, F, px, written);
    }
    // the warp's queued clip items, 32 at a time (no CTA barrier: warps finish on their own):
    // each triangle is clipped and its fan packed two triangles per record
    __syncwarp();
    const uint32_t nclip = s_nclip[warp];
    for (uint32_t r = 0; r < nclip; r += 32) {  // warp-uniform trip count
        const bool has = r + lane < nclip;
        uint32_t pp = 0;
        int f = 0;
        float4 cv[4];
        if (has) {
            const uint32_t it = s_clipq[warp][r + lane];
            pp = it >> 3;
            f = (int)(it & 7u);
            float q[12];
            load_quad(verts, pp, q);
            face_corners(q, s_mvp + f * 16, f, cv);
        }
        const FaceInfo& F = g.face[f];
        const float hw = 0.5f * (float)F.vp[2], hh = 0.5f * (float)F.vp[3];
        const float vx = (float)F.vp[0], vy = (float)F.vp[1];
        for (int t = 0; t < 2; t++) {
            float4 poly[12];
            int pn = 0;
            if (has) {
                poly[0] = cv[0];
                poly[1] = cv[1 + t];
                poly[2] = cv[2 + t];
                pn = clip_polygon(poly, 3);
            }
            const uint32_t ncand = fan_records(pn);
            const uint32_t base = warp_alloc(&b.tri_counts[hi], ncand);
            if (ncand) emit_polygon(g, b, poly, pn, base, pp, hi, f, hw, hh, vx, vy, cnt, st);  // counts its bins
        }
    }
}

void launch_setup(const Geo& g, const Batch& b, const float* verts, const float* gbox, DevState* st,
                  cudaStream_t s) {
    dim3 grid((g.n + 127) / 128, b.K);
    k_setup<<<grid, 128, 0, s>>>(g, b, verts, gbox, st);
}

// ---------------------------------------------------------------------------
// Bin lists
// ---------------------------------------------------------------------------
// Exclusive scan of each hemicube's nb bin counts, one CTA per hemicube (the hemicubes' lists
// have separate regions of list_cap_h references), in tiles of 4 counts per thread: warps scan
// with shuffles, a carry links the tiles.  Also clears the fill cursors and flags a bin-list
// overflow of the hemicube.
__global__ void __launch_bounds__(256) k_scan(Geo g, Batch b, DevState* st) {
    if (st->stopped) return;
    const uint32_t hi = blockIdx.x, total = g.nb;
    uint32_t* count = b.bin_count + (size_t)hi * g.nb;
    uint32_t* offset = b.bin_offset + (size_t)hi * g.nb;
    uint32_t* fill = b.bin_fill + (size_t)hi * g.nb;
    const uint32_t region = hi * b.list_cap_h;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < total; base += 4 * blockDim.x) {
        const uint32_t i0 = base + 4 * tid;
        uint32_t c[4];
#pragma unroll
        for (int k = 0; k < 4; k++) c[k] = i0 + k < total ? count[i0 + k] : 0u;
        const uint32_t t4 = (c[0] + c[1]) + (c[2] + c[3]);
        uint32_t x = t4;  // inclusive warp scan of the threads' 4-count totals
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < nwarps ? s_warp[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= (uint32_t)o) w += y;
            }
            s_warp[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        uint32_t run = s_carry + (warp ? s_warp[warp - 1] : 0u) + (x - t4);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (i0 + k < total) {
                offset[i0 + k] = region + run;
                fill[i0 + k] = 0;
            }
            run += c[k];
        }
        __syncthreads();
        if (tid == blockDim.x - 1) s_carry = run;  // the tile's end
        __syncthreads();
    }
    if (tid == 0 && s_carry > b.list_cap_h) atomicOr(&st->overflow, 2u);
}

__global__ void k_fill(Geo g, Batch b, DevState* st) {
    if (st->stopped) return;
    const uint32_t hi = blockIdx.y;
    const uint32_t ntri = min(b.tri_counts[hi], b.tri_cap_h);
    const TriRec* tris = b.tris + (size_t)hi * b.tri_cap_h;
    const int sh = (int)g.tile_shift;
    const uint32_t lane = threadIdx.x & 31;
    // warp-uniform trip count so that single-bin triangles can be grouped by bin
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t s0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); s0 < ntri; s0 += stride) {
        const uint32_t s = s0 + lane;
        const uint32_t gs = hi * b.tri_cap_h + s;  // batch-wide record index
        bool on = s < ntri;
        int c0 = 0, c1 = -1, r0 = 0, r1 = -1;
        size_t gb0 = 0;
        uint32_t bins_x = 0;
        if (on) {
            const int4 tail = *reinterpret_cast<const int4*>(&tris[s].ay[1]);  // ay[1], id, bx, by
            on = (uint32_t)tail.y != kDeadTri;
            if (on) {
                TriRec t;
                t.bx = (uint32_t)tail.z;
                t.by = (uint32_t)tail.w;
                const FaceInfo& F = g.face[rec_face(t)];
                c0 = (rec_px0(t) - F.sc[0]) >> sh;
                c1 = (rec_px1(t) - F.sc[0]) >> sh;
                r0 = (rec_py0(t) - F.sc[1]) >> sh;
                r1 = (rec_py1(t) - F.sc[1]) >> sh;
                gb0 = (size_t)hi * g.nb + F.bin_base;
                bins_x = F.bins_x;
            }
        }
        const bool single = on && c0 == c1 && r0 == r1;
        const size_t gb1 = gb0 + (size_t)r0 * bins_x + c0;
        const unsigned long long key = single ? (unsigned long long)gb1 : ~0ull;
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        if (single) {
            const int leader = __ffs(grp) - 1;
            uint32_t pos = 0;
            if ((int)lane == leader) pos = atomicAdd(&b.bin_fill[gb1], (uint32_t)__popc(grp));
            pos = __shfl_sync(grp, pos, leader) + __popc(grp & ((1u << lane) - 1u));
            const uint32_t idx = b.bin_offset[gb1] + pos;
            if (idx < b.list_cap) b.bin_list[idx] = gs;
        } else if (on) {
            for (int r = r0; r <= r1; r++)
                for (int c = c0; c <= c1; c++) {
                    const size_t gb = gb0 + (size_t)r * bins_x + c;
                    const uint32_t pos = atomicAdd(&b.bin_fill[gb], 1u);
                    const uint32_t idx = b.bin_offset[gb] + pos;
                    if (idx < b.list_cap) b.bin_list[idx] = gs;
                }
        }
    }
}

void launch_bins(const Geo& g, const Batch& b, DevState* st, cudaStream_t s) {
    k_scan<<<b.K, 256, 0, s>>>(g, b, st);
    k_fill<<<dim3(std::max(2u, (152u * 16u) / b.K), b.K), 256, 0, s>>>(g, b, st);
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

// ff * 2^61 as an integer, exactly, for a delta form factor ff (an integer multiple of 2^-61
// below 1; zero for zero): the float's significand shifted by its exponent, with integer
// instructions only (no 64-bit conversion unit).
__device__ __forceinline__ unsigned long long ff_fixed61(float ff) {
    const uint32_t bits = __float_as_uint(ff);
    if (bits == 0u) return 0ull;
    const unsigned long long m = (unsigned long long)((bits & 0x7FFFFFu) | 0x800000u);
    const int sh = (int)(bits >> 23) - 89;  // ff * 2^61 = m * 2^(e - 127 - 23 + 61)
    return sh >= 0 ? m << sh : m >> -sh;
}

// Exact warp-segmented sum of q over lanes sharing `key`; returns the group's sum
// on every lane and the group mask in *gm.
__device__ __forceinline__ unsigned long long group_sum(unsigned long long key, unsigned long long q, unsigned* gm) {
    unsigned m = __match_any_sync(0xffffffffu, key);
    uint32_t a = (uint32_t)(q & 0x1FFFFFull), bb = (uint32_t)((q >> 21) & 0x1FFFFFull), c = (uint32_t)(q >> 42);
    uint32_t sa = __reduce_add_sync(m, a), sb = __reduce_add_sync(m, bb), sc = __reduce_add_sync(m, c);
    *gm = m;
    return (unsigned long long)sa + ((unsigned long long)sb << 21) + ((unsigned long long)sc << 42);
}

constexpr int32_t kSmallExtent = 16384;  // 64 px in 24.8 fixed point: edge values fit int32

// A big record's parts the warp path needs (68 bytes in shared memory): the two triangles
// A = (v0,v1,v2), B = (v0,v2,v3) with their depth planes.
struct RQuad {
    int32_t X[4], Y[4];
    float c0[2], ax[2], ay[2];
    uint32_t id, flags;  // flags: kRecA | kRecB
    uint32_t pad;
};
// One triangle, for the warp path.
struct RTri {
    int32_t X[3], Y[3];
    float c0, ax, ay;
    uint32_t id;
};

__device__ __forceinline__ bool inside_edge(long long e, bool tl) { return e > 0 || (e == 0 && tl); }

// Exclusive prefix sum of v over a 256-thread block; returns this thread's offset and
// leaves the block total in ws[8].  Contains two __syncthreads.
__device__ __forceinline__ int block_exclusive_scan(int v, uint32_t* ws) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = (uint32_t)x;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int k = 0; k < 8; k++) {
            const uint32_t t = ws[k];
            ws[k] = run;
            run += t;
        }
        ws[8] = run;
    }
    __syncthreads();
    return (int)ws[warp] + x - v;
}

// Triangle A (which = 0) or B (which = 1) of a record, for the warp path.
__device__ __forceinline__ RTri rec_tri(const RQuad& q, int which) {
    RTri t;
    t.X[0] = q.X[0];
    t.Y[0] = q.Y[0];
    t.X[1] = q.X[1 + which];
    t.Y[1] = q.Y[1 + which];
    t.X[2] = q.X[2 + which];
    t.Y[2] = q.Y[2 + which];
    t.c0 = q.c0[which];
    t.ax = q.ax[which];
    t.ay = q.ay[which];
    t.id = q.id;
    return t;
}

// One warp rasterises a large triangle in 8x4 stamps.  The 32 lanes first
// classify 32 stamps at a time against the three edges (wholly outside one edge:
// skipped; wholly inside all edges: no per-pixel edge test), then the warp walks
// only the surviving stamps, one pixel per lane.  Edge values are exact int64.
template <int TILE>
__device__ __forceinline__ void raster_big(const RTri& t, int x0, int x1, int y0, int y1, const BinInfo& bi, int sx,
                                           int sy, unsigned long long* key, int lane, uint32_t* cnt) {
    long long eo[3], stx[3], sty[3], off[3];
    bool tl[3];
    const int lx = lane & 7, ly = lane >> 3;
    long long mx[3], mn[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int j = k == 2 ? 0 : k + 1;
        const long long dx = (long long)t.X[j] - t.X[k], dy = (long long)t.Y[j] - t.Y[k];
        eo[k] = dx * ((long long)y0 * 256 + 128 - t.Y[k]) - dy * ((long long)x0 * 256 + 128 - t.X[k]);
        stx[k] = -dy * 256;
        sty[k] = dx * 256;
        off[k] = stx[k] * lx + sty[k] * ly;
        mx[k] = (stx[k] > 0 ? stx[k] * 7 : 0) + (sty[k] > 0 ? sty[k] * 3 : 0);
        mn[k] = (stx[k] < 0 ? stx[k] * 7 : 0) + (sty[k] < 0 ? sty[k] * 3 : 0);
        tl[k] = (t.Y[j] < t.Y[k]) || (t.Y[j] == t.Y[k] && t.X[j] < t.X[k]);
    }
    const int nsx = (x1 - x0 + 8) >> 3, nsy = (y1 - y0 + 4) >> 2, nst = nsx * nsy;
    uint32_t visited = 0, accepted = 0, plotted = 0;
    for (int base = 0; base < nst; base += 32) {
        const int s = base + lane;
        long long es[3] = {0, 0, 0};
        bool live = false, acc = false;
        int mcx = 0, mcy = 0;
        if (s < nst) {
            mcy = s / nsx;
            mcx = (s - mcy * nsx) * 8;
            mcy *= 4;
            const long long cx = mcx, cy = mcy;
            live = true;
            acc = true;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                es[k] = eo[k] + stx[k] * cx + sty[k] * cy;
                if (es[k] + mx[k] < 0) live = false;
                if (!(es[k] + mn[k] > 0)) acc = false;
            }
        }
        const unsigned lm = __ballot_sync(0xffffffffu, live), am = __ballot_sync(0xffffffffu, live && acc);
        visited += __popc(lm);
        accepted += __popc(am);
        // live stamps two at a time: the two pixel tests of a lane are independent
        unsigned todo = lm;
        while (todo) {
            const int j1 = __ffs(todo) - 1;
            todo &= todo - 1;
            const int j2 = todo ? __ffs(todo) - 1 : j1;
            const bool two = todo != 0;
            todo &= todo - 1;
            const int pxa = x0 + __shfl_sync(0xffffffffu, mcx, j1) + lx, pya = y0 + __shfl_sync(0xffffffffu, mcy, j1) + ly;
            const int pxb = x0 + __shfl_sync(0xffffffffu, mcx, j2) + lx, pyb = y0 + __shfl_sync(0xffffffffu, mcy, j2) + ly;
            const long long a0 = __shfl_sync(0xffffffffu, es[0], j1), a1 = __shfl_sync(0xffffffffu, es[1], j1),
                            a2 = __shfl_sync(0xffffffffu, es[2], j1);
            const long long b0 = __shfl_sync(0xffffffffu, es[0], j2), b1 = __shfl_sync(0xffffffffu, es[1], j2),
                            b2 = __shfl_sync(0xffffffffu, es[2], j2);
            bool ina = pxa <= x1 && pya <= y1;
            bool inb = two && pxb <= x1 && pyb <= y1;
            if (ina && !((am >> j1) & 1u))
                ina = inside_edge(a0 + off[0], tl[0]) && inside_edge(a1 + off[1], tl[1]) &&
                      inside_edge(a2 + off[2], tl[2]);
            if (inb && !((am >> j2) & 1u))
                inb = inside_edge(b0 + off[0], tl[0]) && inside_edge(b1 + off[1], tl[1]) &&
                      inside_edge(b2 + off[2], tl[2]);
            if (ina) {
                const float u = (float)(pxa - sx), w = (float)(pya - sy);
                const float D = (t.c0 + t.ax * u) + t.ay * w;
                atomicMin(&key[(pya - bi.y0) * TILE + (pxa - bi.x0)], ((unsigned long long)depth_ordinal(D) << 32) | t.id);
                plotted++;
            }
            if (inb) {
                const float u = (float)(pxb - sx), w = (float)(pyb - sy);
                const float D = (t.c0 + t.ax * u) + t.ay * w;
                atomicMin(&key[(pyb - bi.y0) * TILE + (pxb - bi.x0)], ((unsigned long long)depth_ordinal(D) << 32) | t.id);
                plotted++;
            }
        }
    }
    if (cnt && lane == 0) {
        atomicAdd(&cnt[4], (uint32_t)nst);
        atomicAdd(&cnt[5], visited);
        atomicAdd(&cnt[6], accepted);
    }
    if (cnt) atomicAdd(&cnt[7], plotted);
}

// The big records of a chunk: one warp per triangle of a record (A, then B).  Record i is
// the RQuad at recs + i * stride bytes.
// The big records of a chunk: one warp per triangle of a record (A, then B).  Record i is
// the RQuad at recs + i * stride bytes.
template <int TILE>
__device__ __forceinline__ void raster_big_records(const unsigned char* recs, int stride, const uint8_t* bigi,
                                                   int nbig, const BinInfo& bi, int sx, int sy,
                                                   unsigned long long* key, int lane, uint32_t* ctr) {
    const int bx1 = bi.x0 + bi.w - 1, by1 = bi.y0 + bi.h - 1;
    for (int i = (int)(threadIdx.x >> 5); i < 2 * nbig; i += (int)(blockDim.x >> 5)) {
        const RQuad& q = *reinterpret_cast<const RQuad*>(recs + (size_t)bigi[i >> 1] * stride);
        const int which = i & 1;
        if (!(q.flags & (which ? kRecB : kRecA))) continue;
        const RTri t = rec_tri(q, which);
        const int32_t xmn = min(t.X[0], min(t.X[1], t.X[2])), xmx = max(t.X[0], max(t.X[1], t.X[2]));
        const int32_t ymn = min(t.Y[0], min(t.Y[1], t.Y[2])), ymx = max(t.Y[0], max(t.Y[1], t.Y[2]));
        const int x0 = max((int)floordiv256((long long)xmn - 128 + 255), (int)bi.x0);
        const int x1 = min((int)floordiv256((long long)xmx - 128), bx1);
        const int y0 = max((int)floordiv256((long long)ymn - 128 + 255), (int)bi.y0);
        const int y1 = min((int)floordiv256((long long)ymx - 128), by1);
        if (x0 <= x1 && y0 <= y1) raster_big<TILE>(t, x0, x1, y0, y1, bi, sx, sy, key, lane, ctr);
    }
}

// The end of a bin, after its records are rasterised (all threads): the counters, the item
// buffer (write_items) and the fused reduction (fused).  For the reduction each thread walks
// kSeg pixels down one column of the bin, summing the exact fixed-point delta form factors
// (ff * 2^61, integers) while the patch id stays the same, and adds each run's sum to the
// hemicube's row with one 64-bit atomic.  Integer sums commute, so the row is exact and
// independent of the order of the adds.  Lanes take adjacent columns (conflict-free key
// reads, coalesced table reads).
template <int TILE>
__host__ __device__ constexpr int finish_seg() { return TILE * TILE / 256 > 4 ? TILE * TILE / 256 : 4; }  // pixels per walker

// The walker's column segment of the bin's delta form factors (an L2-resident table).
template <int TILE>
__device__ __forceinline__ void finish_load(const Geo& g, const float* __restrict__ fftab, const BinInfo& bi,
                                            bool walker, float* ffv) {
    constexpr int kSeg = finish_seg<TILE>();
    const int wx = threadIdx.x % TILE, wr0 = (threadIdx.x / TILE) * kSeg;
#pragma unroll
    for (int i = 0; i < kSeg; i++) {
        ffv[i] = 0.f;
        if (walker && wx < bi.w && wr0 + i < bi.h) ffv[i] = fftab[(size_t)(bi.y0 + wr0 + i) * g.TW + bi.x0 + wx];
    }
}

// Called after a barrier that follows the bin's last key update (all threads).
template <int TILE>
__device__ __forceinline__ void raster_finish(const Geo& g, const Batch& b, DevState* st, int write_items,
                                              int count, uint32_t gb, uint32_t hi, const BinInfo& bi, bool valid,
                                              bool walker, const float* ffv, const unsigned long long* key,
                                              const uint32_t* s_cnt) {
    constexpr int kSeg = finish_seg<TILE>();
    const int wx = threadIdx.x % TILE, wr0 = (threadIdx.x / TILE) * kSeg;
    if (count && threadIdx.x < 8) {
        uint32_t v = s_cnt[threadIdx.x];
        if (threadIdx.x == 0) v = valid ? min(b.bin_count[gb], b.list_cap) : 0u;
        if (v) atomicAdd(&st->raster_counters[threadIdx.x], (unsigned long long)v);
    }
    if (write_items) {
        const size_t img = (size_t)hi * g.RES;
        for (int j = threadIdx.x; j < TILE * TILE; j += blockDim.x) {
            const int ly = j / TILE, lx = j % TILE;
            if (lx >= bi.w || ly >= bi.h) continue;
            const unsigned long long k = key[j];
            const bool has = valid && k != ~0ull;
            b.items[img + (size_t)(bi.y0 + ly) * g.TW + bi.x0 + lx] = has ? (uint32_t)k + 1u : 0u;
        }
    }
    if (!walker) return;
    unsigned long long* Fq = b.Fq + (size_t)hi * g.n;
    const bool col_in = wx < bi.w;
    uint32_t cur = 0xFFFFFFFFu;
    unsigned long long acc = 0;
#pragma unroll
    for (int i = 0; i < kSeg; i++) {
        const unsigned long long k = key[(wr0 + i) * TILE + wx];
        const bool has = col_in && wr0 + i < bi.h && k != ~0ull;
        const uint32_t id = has ? (uint32_t)k : 0xFFFFFFFFu;
        if (id != cur) {
            if (cur != 0xFFFFFFFFu) atomicAdd(&Fq[cur], acc);
            cur = id;
            acc = 0;
        }
        if (has) acc += ff_fixed61(ffv[i]);
    }
    if (cur != 0xFFFFFFFFu) atomicAdd(&Fq[cur], acc);
}

// Small records: exact row spans, then one packed pixel stream per warp.
//
// A small record (extent <= 64 px and box clamped to the bin <= small_max px) is staged as the
// constants of its five tracked edges at the centre of the top-left pixel of its clamped box,
// so that any row's covered columns follow exactly from integer bounds:
//   f_e(n, r) = f0_e + r * (dx_e * 256) - n * (dy_e * 256)   (column n, row r of the box)
// is the biased edge value E + tl - 1 (E the exact 24.8 edge function, tl the top-left flag;
// inside: f >= 0), and f_e >= 0  <=>  n >= -floor(f_e(0, r) / a_e) when dy_e < 0, or
// n <= floor(f_e(0, r) / a_e) when dy_e > 0, with a_e = |dy_e| * 256; a horizontal edge
// (dy_e = 0) admits the whole row or none of it.  Triangle A is edges 0, 1, 2 (v0->v1,
// v1->v2, v2->v0); B is v0->v2, 3 and 4 (v2->v3, v3->v0), where v0->v2 is the complement of
// edge 2 (f = -f_2 - 1, so floor(f / a) = -floor(f_2 / a) - 1).  A pixel inside both (a
// folded outline) is in both spans and gets both keys, the smaller winning, as two draws would.
struct SpanRec {
    int32_t f0[5];   // biased edge values at the centre of the box's top-left pixel
    uint32_t dxy[5]; // (uint16) dx | dy << 16, 24.8 edge vector (|dx|, |dy| <= 16384)
    float pl[6];     // c0, ax, ay of A, then of B (constant at the scissor origin; gradients x256)
    uint32_t id;
    uint32_t geo;    // x0 - bin x0 | (w - 1) << 6 | y0 - bin y0 << 12 | A << 18 | B << 19
};
static_assert(sizeof(SpanRec) == 72 && sizeof(RQuad) <= sizeof(SpanRec), "staging slot");
constexpr int kSpanChunk = 256;    // records staged per CTA round (indices stored as uint8)
constexpr int kRowCap = 2048;      // rows per pass over a chunk's small records
constexpr int kRegionBytes = kSpanChunk * (int)sizeof(SpanRec);
template <int TILE>
constexpr int raster_dyn_smem() { return TILE * TILE * 8 + kRegionBytes; }

// rcp.approx: relative error about 2^-23, which the exact integer step of floor_div absorbs.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// floor(f / a) for a > 0 (a multiple of 256, at most 2^22) where only results in [-65, 65]
// matter exactly: a float estimate (relative error a few 2^-24, so off by at most one inside
// the clamp), clamped, then one exact integer correction.  Outside the clamp the result keeps
// the right side of [-65, 65], which is all the span bounds need.
__device__ __forceinline__ int32_t floor_div(int32_t f, int32_t a) {
    const float q = __int2float_rn(f) * rcp_approx(__int2float_rn(a));
    int32_t m = max(-66, min(66, __float2int_rd(q)));
    const int32_t r = f - m * a;  // in [0, a) exactly when m is the floor
    return m + (r >= a ? 1 : 0) - (r < 0 ? 1 : 0);
}

// The bound one edge puts on its triangle's span [lo, hi] in a row; lo starts at 0 and hi at
// w - 1 <= 63, so 0 and 64 are neutral.
__device__ __forceinline__ void edge_bound(int32_t f, int32_t dy, int& lo, int& hi) {
    const int32_t m = floor_div(f, max(abs(dy) * 256, 256));
    lo = max(lo, dy < 0 ? -m : 0);
    hi = min(hi, dy > 0 ? m : ((dy == 0 && f < 0) ? -1 : 64));
}

// CTA per (hemicube, TILE x TILE bin), 256 threads, records in chunks of kSpanChunk:
//  1. each thread stages one record: a small one as a SpanRec, a big one as an RQuad;
//  2. a block scan numbers the small records' rows, and row items are mapped to records;
//  3. warps take 32 rows at a time from a shared cursor: each lane computes its row's spans
//     of A and B, the warp lays the spans' pixels out as one stream, and each lane then takes
//     one pixel of every 32 (it finds its span through a bit mask of span starts), evaluates
//     the depth plane and does a 64-bit atomicMin of depth|id into the bin's keys;
//  4. big records (extent > 64 px or a box above small_max), one warp per triangle;
// then raster_finish.  PROF adds SM-cycle counters per phase (raster counters 8..15); it is
// launched only for phase profiling.
template <int TILE, bool PROF>
__global__ void __launch_bounds__(256, 4) k_raster(Geo g, Batch b, const float* __restrict__ fftab,
                                                   DevState* st, int write_items, int fused, int count) {
    if (st->stopped) return;
    __shared__ unsigned long long s_cyc[8];
    long long tmark = PROF ? clock64() : 0;
    auto mark = [&](int ph) {
        if (PROF) {
            const long long t = clock64();
            if ((threadIdx.x & 31) == 0) atomicAdd(&s_cyc[ph], (unsigned long long)(t - tmark));
            tmark = t;
        }
    };
    if (PROF && threadIdx.x < 8) s_cyc[threadIdx.x] = 0;
    const uint32_t gb = blockIdx.x;
    const uint32_t hi = gb / g.nb, bin = gb % g.nb;
    const BinInfo bi = b.bins[bin];
    const bool valid = b.valid[hi] != 0;
    // dynamic shared memory: the bin's depth|id keys, then the chunk's staged records
    extern __shared__ __align__(16) unsigned char s_dyn[];
    unsigned long long* key = reinterpret_cast<unsigned long long*>(s_dyn);
    unsigned char* s_region = s_dyn + TILE * TILE * 8;
    SpanRec* s_rec = reinterpret_cast<SpanRec*>(s_region);
    __shared__ uint8_t s_bigi[kSpanChunk];       // big records of the chunk
    __shared__ uint16_t s_rowbase[kSpanChunk];   // first row item of each small record
    __shared__ uint8_t s_rowown[kRowCap];        // row item -> record (this pass)
    __shared__ uint32_t s_seg[8][64];            // per warp: the spans of its 32 rows, in stream order
    __shared__ uint32_t s_wsum[9];
    __shared__ int s_nbig;
    __shared__ int s_next;                       // next unclaimed block of 32 rows
    __shared__ uint32_t s_cnt[8];
    uint32_t* ctr = count ? s_cnt : nullptr;
    if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_next = 8 * 32;
    uint32_t cnt = 0, off = 0;
    if (valid) {
        cnt = b.bin_count[gb];
        off = b.bin_offset[gb];
        if (off >= b.list_cap) cnt = 0;
        else if (off + cnt > b.list_cap) cnt = b.list_cap - off;
    }
    // the first chunk's records are requested before the keys are cleared, so that their
    // DRAM latency overlaps the clear
    const bool pre = threadIdx.x < min(cnt, (uint32_t)kSpanChunk);
    int4 pr0 = make_int4(0, 0, 0, 0), pr1 = pr0, pr2 = pr0, pr3 = pr0;
    if (pre) {
        const int4* tr = reinterpret_cast<const int4*>(&b.tris[b.bin_list[off + threadIdx.x]]);
        pr0 = tr[0];
        pr1 = tr[1];
        pr2 = tr[2];
        pr3 = tr[3];
    }
    for (int j = threadIdx.x; j < TILE * TILE; j += blockDim.x) key[j] = ~0ull;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u, le = lt | (1u << lane);
    __syncthreads();
    mark(0);
    const bool walker = fused && valid && (int)threadIdx.x < TILE * TILE / finish_seg<TILE>();
    if (valid) {
        const FaceInfo& F = g.face[bi.face];
        const int sx = F.sc[0], sy = F.sc[1];
        const int ux = bi.x0 - sx, uy = bi.y0 - sy;  // bin origin relative to the scissor origin
        const int bx1 = bi.x0 + bi.w - 1, by1 = bi.y0 + bi.h - 1;
        for (uint32_t base = 0; base < cnt; base += kSpanChunk) {
            const uint32_t m = min((uint32_t)kSpanChunk, cnt - base);
            if (threadIdx.x == 0) s_nbig = 0;
            __syncthreads();
            // 1. load, clamp to the bin, stage: small records as SpanRec, big ones as RQuad
            int rows = 0;
            if (threadIdx.x < m) {
                int4 xs = pr0, ys = pr1, p = pr2, q = pr3;  // q = ay[1], id, bx, by
                if (base != 0) {
                    const int4* tr = reinterpret_cast<const int4*>(&b.tris[b.bin_list[off + base + threadIdx.x]]);
                    xs = tr[0];
                    ys = tr[1];
                    p = tr[2];
                    q = tr[3];
                }
                const int px0 = q.z & 0xFFF, px1 = (q.z >> 12) & 0xFFF;
                const int py0 = q.w & 0xFFF, py1 = (q.w >> 12) & 0xFFF;
                const int x0 = max(px0, (int)bi.x0), x1 = min(px1, bx1);
                const int y0 = max(py0, (int)bi.y0), y1 = min(py1, by1);
                if (x0 <= x1 && y0 <= y1) {
                    const int32_t X[4] = {xs.x, xs.y, xs.z, xs.w}, Y[4] = {ys.x, ys.y, ys.z, ys.w};
                    // the planes' constant terms at the scissor origin, rebuilt with the
                    // set-up's float operations (gx = ax / 256 exactly)
                    const float d0 = __int_as_float(p.x);
                    const float ox = (float)(sx * 256 + 128 - xs.x);  // < 2^29 in magnitude: int32
                    const float oy = (float)(sy * 256 + 128 - ys.x);
                    const float axA = __int_as_float(p.y), axB = __int_as_float(p.z);
                    const float ayA = __int_as_float(p.w), ayB = __int_as_float(q.x);
                    const float c0A = (d0 + (axA * 0x1p-8f) * ox) + (ayA * 0x1p-8f) * oy;
                    const float c0B = (d0 + (axB * 0x1p-8f) * ox) + (ayB * 0x1p-8f) * oy;
                    const uint32_t flags = (uint32_t)q.z & (kRecA | kRecB);
                    const int32_t ex = max(max(X[0], X[1]), max(X[2], X[3])) - min(min(X[0], X[1]), min(X[2], X[3]));
                    const int32_t ey = max(max(Y[0], Y[1]), max(Y[2], Y[3])) - min(min(Y[0], Y[1]), min(Y[2], Y[3]));
                    const int area = (x1 - x0 + 1) * (y1 - y0 + 1);
                    if (ex <= kSmallExtent && ey <= kSmallExtent && area <= (int)g.small_max) {
                        SpanRec& r = s_rec[threadIdx.x];
#pragma unroll
                        for (int k = 0; k < 5; k++) {
                            const int a = k == 0 ? 0 : (k == 1 ? 1 : (k == 2 ? 2 : (k == 3 ? 2 : 3)));  // from
                            const int j = k == 0 ? 1 : (k == 1 ? 2 : (k == 2 ? 0 : (k == 3 ? 3 : 0)));  // to
                            const int32_t dx = X[j] - X[a], dy = Y[j] - Y[a];
                            const bool tl = (Y[j] < Y[a]) || (Y[j] == Y[a] && X[j] < X[a]);
                            r.f0[k] = dx * (y0 * 256 + 128 - Y[a]) - dy * (x0 * 256 + 128 - X[a]) - (tl ? 0 : 1);
                            r.dxy[k] = ((uint32_t)dx & 0xFFFFu) | ((uint32_t)dy << 16);
                        }
                        r.pl[0] = c0A; r.pl[1] = axA; r.pl[2] = ayA;
                        r.pl[3] = c0B; r.pl[4] = axB; r.pl[5] = ayB;
                        r.id = (uint32_t)q.y;
                        r.geo = (uint32_t)(x0 - bi.x0) | ((uint32_t)(x1 - x0) << 6) | ((uint32_t)(y0 - bi.y0) << 12) |
                                ((flags & kRecA) ? 1u << 18 : 0u) | ((flags & kRecB) ? 1u << 19 : 0u);
                        rows = y1 - y0 + 1;
                        if (ctr) {
                            atomicAdd(&ctr[1], 1u);
                            atomicAdd(&ctr[2], (uint32_t)area);
                        }
                    } else {
                        RQuad& t = *reinterpret_cast<RQuad*>(&s_rec[threadIdx.x]);
#pragma unroll
                        for (int k = 0; k < 4; k++) t.X[k] = X[k], t.Y[k] = Y[k];
                        t.c0[0] = c0A; t.c0[1] = c0B;
                        t.ax[0] = axA; t.ax[1] = axB;
                        t.ay[0] = ayA; t.ay[1] = ayB;
                        t.id = (uint32_t)q.y;
                        t.flags = flags;
                        s_bigi[atomicAdd(&s_nbig, 1)] = (uint8_t)threadIdx.x;
                        if (ctr) atomicAdd(&ctr[3], 1u);
                    }
                }
            }
            // 2. row items: record t owns rows [rowbase, rowbase + rows) of the chunk
            const int rowbase = block_exclusive_scan(rows, s_wsum);  // syncs; s_wsum[8] = total
            const int nrows = (int)s_wsum[8];
            mark(1);
            if (rows) s_rowbase[threadIdx.x] = (uint16_t)rowbase;
            for (int pass = 0; pass < nrows; pass += kRowCap) {
                const int np = min(kRowCap, nrows - pass);
                {
                    const int r0 = max(rowbase, pass), r1 = min(rowbase + rows, pass + np);
                    for (int i = r0; i < r1; i++) s_rowown[i - pass] = (uint8_t)threadIdx.x;
                }
                __syncthreads();
                mark(2);
                // 3. blocks of 32 rows: spans of A and B, then their pixels as one stream
                uint32_t* seg = s_seg[warp];
                for (int rb = warp * 32; rb < np;) {  // warp-uniform
                    const int i = rb + lane;
                    int lenA = 0, lenB = 0, loA = 0, loB = 0, yl = 0, xl0 = 0, k = 0;
                    if (i < np) {
                        k = s_rowown[i];
                        const SpanRec& R = s_rec[k];
                        const int r = pass + i - (int)s_rowbase[k];
                        const uint32_t geo = R.geo;
                        xl0 = (int)(geo & 63u);
                        const int w = (int)((geo >> 6) & 63u) + 1;
                        yl = (int)((geo >> 12) & 63u) + r;
                        int32_t f[5], dy[5];
#pragma unroll
                        for (int e = 0; e < 5; e++) {
                            const uint32_t d = R.dxy[e];
                            const int32_t dx = (int32_t)(int16_t)(d & 0xFFFFu);
                            dy[e] = (int32_t)(int16_t)(d >> 16);
                            f[e] = R.f0[e] + r * (dx * 256);
                        }
                        int hiA = w - 1, hiB = w - 1;
                        edge_bound(f[0], dy[0], loA, hiA);
                        edge_bound(f[1], dy[1], loA, hiA);
                        edge_bound(f[3], dy[3], loB, hiB);
                        edge_bound(f[4], dy[4], loB, hiB);
                        // edge 2 bounds A; its complement v0->v2 bounds B
                        const int32_t m2 = floor_div(f[2], max(abs(dy[2]) * 256, 256));
                        loA = max(loA, dy[2] < 0 ? -m2 : 0);
                        hiA = min(hiA, dy[2] > 0 ? m2 : ((dy[2] == 0 && f[2] < 0) ? -1 : 64));
                        loB = max(loB, dy[2] > 0 ? m2 + 1 : 0);
                        hiB = min(hiB, dy[2] < 0 ? -m2 - 1 : ((dy[2] == 0 && f[2] >= 0) ? -1 : 64));
                        if (geo & (1u << 18)) lenA = max(0, hiA - loA + 1);
                        if (geo & (1u << 19)) lenB = max(0, hiB - loB + 1);
                    }
                    // stream offsets of this lane's pixels (warp exclusive scan)
                    const int n = lenA + lenB;
                    int x = n;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int y = __shfl_up_sync(0xffffffffu, x, o);
                        if (lane >= o) x += y;
                    }
                    const int total = __shfl_sync(0xffffffffu, x, 31);
                    const int sA = x - n, sB = sA + lenA;
                    // span table in stream order: rank = non-empty spans of the lower lanes;
                    // entry: (start - first column + 64) | row << 13 | triangle << 19 | record << 20
                    const unsigned bA = __ballot_sync(0xffffffffu, lenA > 0), bB = __ballot_sync(0xffffffffu, lenB > 0);
                    const int rank = __popc(bA & lt) + __popc(bB & lt);
                    if (lenA > 0) seg[rank] = (uint32_t)(sA - (xl0 + loA) + 64) | ((uint32_t)yl << 13) | ((uint32_t)k << 20);
                    if (lenB > 0)
                        seg[rank + (lenA > 0)] =
                            (uint32_t)(sB - (xl0 + loB) + 64) | ((uint32_t)yl << 13) | (1u << 19) | ((uint32_t)k << 20);
                    __syncwarp();
                    mark(3);
                    int S = 0;  // spans that start before the window
                    for (int w0 = 0; w0 < total; w0 += 32) {
                        uint32_t bits = 0;
                        if (lenA > 0 && (unsigned)(sA - w0) < 32u) bits |= 1u << (sA - w0);
                        if (lenB > 0 && (unsigned)(sB - w0) < 32u) bits |= 1u << (sB - w0);
                        const unsigned starts = __reduce_or_sync(0xffffffffu, bits);
                        const int gpos = w0 + lane;
                        if (gpos < total) {
                            const uint32_t e = seg[S + __popc(starts & le) - 1];
                            const int xl = gpos - ((int)(e & 0x1FFFu) - 64);
                            const int ylf = (int)((e >> 13) & 63u);
                            const SpanRec& R = s_rec[e >> 20];
                            const float* pl = R.pl + 3 * ((e >> 19) & 1u);
                            const float u = (float)(ux + xl), wv = (float)(uy + ylf);
                            const float D = (pl[0] + pl[1] * u) + pl[2] * wv;
                            atomicMin(&key[ylf * TILE + xl], ((unsigned long long)depth_ordinal(D) << 32) | R.id);
                        }
                        S += __popc(starts);
                    }
                    __syncwarp();
                    mark(4);
                    if (lane == 0) rb = atomicAdd(&s_next, 32);
                    rb = __shfl_sync(0xffffffffu, rb, 0);
                }
                // after the last pass of the last chunk the warps go straight on to the big
                // records (the chunk barrier below orders them before the bin end)
                if (!(pass + np >= nrows && base + kSpanChunk >= cnt)) {
                    __syncthreads();
                    if (threadIdx.x == 0) s_next = 8 * 32;
                }
                mark(5);
            }
            // 4. big records: one warp per triangle
            raster_big_records<TILE>(s_region, (int)sizeof(SpanRec), s_bigi, s_nbig, bi, sx, sy, key, lane, ctr);
            __syncthreads();
            mark(6);
        }
    }
    // the walkers' delta form factors (loading them any earlier keeps 16 registers live through
    // the big-record path, whose 64-bit edge arithmetic then spills)
    float ffv[finish_seg<TILE>()];
    finish_load<TILE>(g, fftab, bi, walker, ffv);
    raster_finish<TILE>(g, b, st, write_items, count, gb, hi, bi, valid, walker, ffv, key, s_cnt);
    if (PROF) {
        mark(7);
        __syncthreads();
        if (threadIdx.x < 8) atomicAdd(&st->raster_counters[8 + threadIdx.x], s_cyc[threadIdx.x]);
    }
}

template <int TILE, bool PROF>
static cudaError_t raster_attrs() {
    cudaError_t e = cudaFuncSetAttribute(k_raster<TILE, PROF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         raster_dyn_smem<TILE>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_raster<TILE, PROF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    return e;
}

cudaError_t raster_init() {
    cudaError_t e = raster_attrs<16, false>();
    if (e == cudaSuccess) e = raster_attrs<32, false>();
    if (e == cudaSuccess) e = raster_attrs<64, false>();
    if (e == cudaSuccess) e = raster_attrs<16, true>();
    if (e == cudaSuccess) e = raster_attrs<32, true>();
    if (e == cudaSuccess) e = raster_attrs<64, true>();
    return e;
}

void launch_raster(const Geo& g, const Batch& b, const float* fftab, DevState* st, bool write_items,
                   bool fused_reduce, cudaStream_t s, bool count, bool phases) {
    dim3 grid(b.K * g.nb);
#define RAD_RASTER_LAUNCH(T, P) \
    k_raster<T, P><<<grid, 256, raster_dyn_smem<T>(), s>>>(g, b, fftab, st, write_items, fused_reduce, count)
    if (phases) {
        if (g.tile == 16) RAD_RASTER_LAUNCH(16, true);
        else if (g.tile == 64) RAD_RASTER_LAUNCH(64, true);
        else RAD_RASTER_LAUNCH(32, true);
    } else {
        if (g.tile == 16) RAD_RASTER_LAUNCH(16, false);
        else if (g.tile == 64) RAD_RASTER_LAUNCH(64, false);
        else RAD_RASTER_LAUNCH(32, false);
    }
#undef RAD_RASTER_LAUNCH
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
    if (has) q = ff_fixed61(fftab[pix]);
    // the lanes of one warp may span several images (an image is 3W^2 texels: 12 at W = 2),
    // so the key carries the whole image index beside the patch id
    const unsigned long long key = has ? ((unsigned long long)hi << 32) | (it - 1) : ~0ull;
    unsigned gm;
    unsigned long long sum = group_sum(key, q, &gm);
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
