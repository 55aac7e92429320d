// C ABI of the solver (include/radiosity.h): context, device memory, batch
// sequencing and the CUDA-graph shoot loop.
//
// One rad_ctx owns one CUDA stream on one device.  A shoot batch is nine
// stream-ordered operations (2 memsets, select, camera, setup, scan, fill,
// raster+reduce, update, emitters); rad_shoot captures one batch into a CUDA
// graph once per context and replays it, checking the device stop flag every
// 32 batches.  Every kernel reads the device stop flag first, so batches after
// the stop rule fired are no-ops and the result equals the reference's early exit.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <unistd.h>
#include <string>
#include <vector>

#include "radiosity.h"
#include "rad_ctx.cuh"
#include "rad_internal.cuh"

namespace rad {
void launch_power0(const float4* rad, const float* area, uint32_t n, DevState* st, cudaStream_t s);
}

using namespace rad;

#define RAD_CUDA(ctx, call)                                                                         \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);                        \
            return e_ == cudaErrorMemoryAllocation ? RAD_E_NOMEM : RAD_E_CUDA;                      \
        }                                                                                           \
    } while (0)

static int fail(rad_ctx* ctx, int code, const char* msg) {
    if (ctx) ctx->err = msg;
    return code;
}
int ctx_fail(rad_ctx* ctx, int code, const char* msg) { return fail(ctx, code, msg); }

template <typename T>
static void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

static void free_batch(BatchBuf& bb) {
    dfree(bb.b.shooters);
    dfree(bb.b.valid);
    dfree(bb.b.saved);
    dfree(bb.b.mvp);
    dfree(bb.b.frame);
    dfree(bb.b.tris);
    dfree(bb.b.bin_count);
    dfree(bb.b.tri_counts);
    dfree(bb.b.bin_offset);
    dfree(bb.b.bin_fill);
    dfree(bb.b.bin_list);
    dfree(bb.b.Fq);
    dfree(bb.b.items);
    dfree(bb.b.sel_hist);
    dfree(bb.b.sel_ctrl);
    dfree(bb.b.sel_keys);
    dfree(bb.b.sel_sure);
    dfree(bb.b.sel_bnd);
    dfree(bb.b.partials);
    bb.cap_k = 0;
    bb.has_items = false;
}

static void free_dense(rad_ctx* c) {
    dfree(c->d_F32);
    dfree(c->d_F16);
    dfree(c->d_scale);
    dfree(c->d_F32T);
    dfree(c->d_F16T);
    dfree(c->d_inv_area);
    dfree(c->d_wT);
    c->dense_ready = false;
    c->dense_shoot = false;
}

static uint32_t tri_cap_per_hemi(const rad_ctx* c) {
    return c->cfg.tri_capacity ? c->cfg.tri_capacity : 3u * c->n + 4096u;
}
static uint32_t list_cap_per_hemi(const rad_ctx* c) {
    return c->cfg.binref_capacity ? c->cfg.binref_capacity : 4u * tri_cap_per_hemi(c);
}

static int alloc_batch(rad_ctx* c, BatchBuf& bb, uint32_t K, bool items);
int ctx_alloc_batch(rad_ctx* c, BatchBuf& bb, uint32_t K, bool items) { return alloc_batch(c, bb, K, items); }
static int alloc_batch(rad_ctx* c, BatchBuf& bb, uint32_t K, bool items) {
    if (bb.cap_k >= K && (!items || bb.has_items) && bb.b.Fq) {
        bb.b.K = K;
        return RAD_OK;
    }
    free_batch(bb);
    Batch& b = bb.b;
    const uint64_t tri_cap = (uint64_t)tri_cap_per_hemi(c) * K, list_cap = (uint64_t)list_cap_per_hemi(c) * K;
    if (tri_cap > 0xFFFFFFF0ull || list_cap > 0xFFFFFFF0ull)
        return fail(c, RAD_E_INVALID, "batch capacity exceeds 2^32 records; lower hemicubes_count");
    b.K = K;
    b.tri_cap = (uint32_t)tri_cap;
    b.tri_cap_h = tri_cap_per_hemi(c);
    b.list_cap = (uint32_t)list_cap;
    b.list_cap_h = list_cap_per_hemi(c);
    const size_t nbk = (size_t)K * c->geo.nb;
    RAD_CUDA(c, cudaMalloc(&b.shooters, sizeof(uint32_t) * K));
    RAD_CUDA(c, cudaMalloc(&b.valid, sizeof(uint32_t) * K));
    RAD_CUDA(c, cudaMalloc(&b.saved, sizeof(float4) * K));
    RAD_CUDA(c, cudaMalloc(&b.mvp, sizeof(float) * 16 * 5 * K));
    RAD_CUDA(c, cudaMalloc(&b.frame, sizeof(float) * 8 * K));
    RAD_CUDA(c, cudaMalloc(&b.tris, sizeof(TriRec) * tri_cap));
    RAD_CUDA(c, cudaMalloc(&b.bin_count, sizeof(uint32_t) * nbk));
    RAD_CUDA(c, cudaMalloc(&b.tri_counts, sizeof(uint32_t) * K));
    RAD_CUDA(c, cudaMalloc(&b.bin_offset, sizeof(uint32_t) * nbk));
    RAD_CUDA(c, cudaMalloc(&b.bin_fill, sizeof(uint32_t) * nbk));
    RAD_CUDA(c, cudaMalloc(&b.bin_list, sizeof(uint32_t) * list_cap));
    RAD_CUDA(c, cudaMalloc(&b.Fq, sizeof(unsigned long long) * (size_t)K * c->n));
    RAD_CUDA(c, cudaMemsetAsync(b.Fq, 0, sizeof(unsigned long long) * (size_t)K * c->n, c->stream));
    RAD_CUDA(c, cudaMemsetAsync(b.valid, 0, sizeof(uint32_t) * K, c->stream));
    if (items) RAD_CUDA(c, cudaMalloc(&b.items, sizeof(uint32_t) * (size_t)K * c->geo.RES));
    RAD_CUDA(c, cudaMalloc(&b.sel_hist, sizeof(uint32_t) * 2048));
    RAD_CUDA(c, cudaMemsetAsync(b.sel_hist, 0, sizeof(uint32_t) * 2048, c->stream));
    RAD_CUDA(c, cudaMalloc(&b.sel_ctrl, sizeof(uint32_t) * 8));
    RAD_CUDA(c, cudaMalloc(&b.sel_keys, sizeof(uint32_t) * c->n));
    RAD_CUDA(c, cudaMalloc(&b.sel_sure, sizeof(unsigned long long) * K));
    RAD_CUDA(c, cudaMalloc(&b.sel_bnd, sizeof(unsigned long long) * c->n));
    RAD_CUDA(c, cudaMalloc(&b.partials, sizeof(double) * kUpdateBlocks));
    b.bins = c->d_bins;
    bb.cap_k = K;
    bb.has_items = items;
    return RAD_OK;
}

static void drop_graph(rad_ctx* c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->graph_exec = nullptr;
    c->graph = nullptr;
}

static void setup_geo(rad_ctx* c, std::vector<BinInfo>& bins) {
    Geo& g = c->geo;
    const uint32_t W = c->cfg.hemicube_side;
    g.W = W;
    g.TW = 2 * W;
    g.TH = (uint32_t)(W * 1.5);
    g.RES = g.TW * g.TH;
    g.mode = c->cfg.mode;
    uint32_t tile = c->cfg.tile;
    if (tile == 0) tile = W >= 512 ? 64 : (W >= 64 ? 32 : 16);
    g.tile = tile;
    g.tile_shift = 0;
    while ((1u << g.tile_shift) < tile) g.tile_shift++;
    g.small_max = c->cfg.small_tri_pixels ? c->cfg.small_tri_pixels : 4096;
    const int w = (int)W, h = (int)W;
    uint32_t base = 0;
    bins.clear();
    for (int f = 0; f < 5; f++) {
        FaceInfo& F = g.face[f];
        F.vp[2] = w;
        F.vp[3] = h;
        switch (f) {  // source/Main.cpp:316-389 with hemicube offset 0
            case 0: F.vp[0] = 0; F.vp[1] = h; break;
            case 1: F.vp[0] = w; F.vp[1] = h / 2; break;
            case 2: F.vp[0] = -1 * (int)(W / 2); F.vp[1] = 0; break;
            case 3: F.vp[0] = (int)(W * 1.5); F.vp[1] = 0; break;
            default: F.vp[0] = w / 2; F.vp[1] = 0; break;
        }
        if (f == 0 || f == 1) {
            F.sc[1] = h;
            F.sc[3] = h / 2;
        } else {
            F.sc[1] = 0;
            F.sc[3] = h;
        }
        F.sc[2] = (f == 2 || f == 3) ? w / 2 : w;
        switch (f) {
            case 0: case 2: F.sc[0] = 0; break;
            case 1: F.sc[0] = w; break;
            case 3: F.sc[0] = (int)(W * 1.5); break;
            default: F.sc[0] = w / 2; break;
        }
        F.bins_x = (F.sc[2] + (int)tile - 1) / (int)tile;
        F.bins_y = (F.sc[3] + (int)tile - 1) / (int)tile;
        F.bin_base = (int)base;
        for (int r = 0; r < F.bins_y; r++)
            for (int cc = 0; cc < F.bins_x; cc++) {
                BinInfo bi;
                bi.x0 = (int16_t)(F.sc[0] + cc * (int)tile);
                bi.y0 = (int16_t)(F.sc[1] + r * (int)tile);
                bi.w = (int16_t)std::min((int)tile, F.sc[0] + F.sc[2] - bi.x0);
                bi.h = (int16_t)std::min((int)tile, F.sc[1] + F.sc[3] - bi.y0);
                bi.face = f;
                bins.push_back(bi);
            }
        base += (uint32_t)(F.bins_x * F.bins_y);
    }
    g.nb = base;
    // Perspective(90, 1.0, 0.01, 1000) -> Frustum (source/Transform.cpp:26-80, source/Main.cpp:1172)
    const float PI = 3.1415926535897932384626433832795028841971691075f;
    float fov = 90, aspect = 1.0f, zn = 0.01f, zf = 1000;
    float fh = (float)(tanf(fov * PI / 180 * .5f)) * zn;
    float fw = fh * aspect;
    float l = -fw, r = fw, bt = -fh, t = fh;
    float* p = g.proj;
    p[0] = 2 * zn / (r - l); p[4] = 0; p[8] = (r + l) / (r - l); p[12] = 0;
    p[1] = 0; p[5] = 2 * zn / (t - bt); p[9] = (t + bt) / (t - bt); p[13] = 0;
    p[2] = 0; p[6] = 0; p[10] = -(zf + zn) / (zf - zn); p[14] = -2 * zf * zn / (zf - zn);
    p[3] = 0; p[7] = 0; p[11] = -1; p[15] = 0;
}

static int check_cfg(const rad_config* cfg) {
    if (!cfg) return RAD_E_INVALID;
    const uint32_t W = cfg->hemicube_side;
    if (W < 2 || W > 2048 || (W & 1u)) return RAD_E_INVALID;
    if (cfg->hemicubes_count < 1 || cfg->hemicubes_count > (uint32_t)kMaxK) return RAD_E_INVALID;
    if (cfg->tile != 0 && cfg->tile != 16 && cfg->tile != 32 && cfg->tile != 64) return RAD_E_INVALID;
    if (cfg->mode > 1) return RAD_E_INVALID;
    if (cfg->ocl_workitems_x == 0) return RAD_E_INVALID;
    if (cfg->small_tri_pixels > 4096) return RAD_E_INVALID;
    return RAD_OK;
}

// One shoot batch on the context stream (graph-capturable: no sync, no alloc).
static void enqueue_batch(rad_ctx* c) {
    Batch& b = c->shoot.b;
    cudaStream_t s = c->stream;
    cudaMemsetAsync(b.tri_counts, 0, sizeof(uint32_t) * b.K, s);
    cudaMemsetAsync(b.bin_count, 0, sizeof(uint32_t) * (size_t)b.K * c->geo.nb, s);
    launch_select(c->geo, b, c->d_rad, c->d_area, c->d_state, s);
    launch_camera(c->geo, b, c->d_verts, c->d_rad, c->d_state, s);
    launch_setup(c->geo, b, c->d_verts, c->d_gbox, c->d_state, s);
    launch_bins(c->geo, b, c->d_state, s);
    launch_raster(c->geo, b, c->d_fftab, c->d_state, false, true, s);
    launch_update(c->geo, b, c->d_color, c->d_rho, c->d_area, c->d_rad, c->d_state, s);
    launch_emitters(c->geo, b, c->d_rad, c->d_illum, c->d_area, c->cfg.tolerance, nullptr, c->d_state, s);
}

// Render (and optionally reduce) `count` given shooters with the aux batch.
static int run_aux(rad_ctx* c, const uint32_t* shooters, uint32_t count, bool items, bool fused) {
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (!shooters || count == 0) return fail(c, RAD_E_INVALID, "no shooters");
    for (uint32_t i = 0; i < count; i++)
        if (shooters[i] >= c->n) return fail(c, RAD_E_INVALID, "shooter index out of range");
    int rc = alloc_batch(c, c->aux, count, items);
    if (rc) return rc;
    Batch& b = c->aux.b;
    b.K = count;
    cudaStream_t s = c->stream;
    std::vector<uint32_t> ones(count, 1u);
    RAD_CUDA(c, cudaMemsetAsync(c->d_aux, 0, sizeof(DevState), s));
    RAD_CUDA(c, cudaMemcpyAsync(b.shooters, shooters, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s));
    RAD_CUDA(c, cudaMemcpyAsync(b.valid, ones.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s));
    RAD_CUDA(c, cudaMemsetAsync(b.tri_counts, 0, sizeof(uint32_t) * count, s));
    RAD_CUDA(c, cudaMemsetAsync(b.bin_count, 0, sizeof(uint32_t) * (size_t)count * c->geo.nb, s));
    RAD_CUDA(c, cudaMemsetAsync(b.Fq, 0, sizeof(unsigned long long) * (size_t)count * c->n, s));
    launch_camera(c->geo, b, c->d_verts, c->d_rad, c->d_aux, s);
    launch_setup(c->geo, b, c->d_verts, c->d_gbox, c->d_aux, s);
    launch_bins(c->geo, b, c->d_aux, s);
    launch_raster(c->geo, b, c->d_fftab, c->d_aux, items, fused, s);
    RAD_CUDA(c, cudaGetLastError());
    DevState st;
    RAD_CUDA(c, cudaMemcpyAsync(&st, c->d_aux, sizeof(st), cudaMemcpyDeviceToHost, s));
    RAD_CUDA(c, cudaStreamSynchronize(s));
    if (st.overflow) return fail(c, RAD_E_OVERFLOW, "triangle or bin capacity exceeded");
    return RAD_OK;
}

static int ensure_rows(rad_ctx* c, size_t count) {
    if (c->rows_cap >= count) return RAD_OK;
    dfree(c->d_rows);
    RAD_CUDA(c, cudaMalloc(&c->d_rows, sizeof(float) * count));
    c->rows_cap = count;
    return RAD_OK;
}

extern "C" {

int rad_config_default(rad_config* cfg) {
    if (!cfg) return RAD_E_INVALID;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->hemicube_side = 16;      // source/Config.cpp:6-10
    cfg->ocl_workitems_x = 4;
    cfg->shoots_per_cycle = 500;
    cfg->max_patch_area = 0.5;
    cfg->hemicubes_count = 10;
    cfg->mode = RAD_MODE_REF;
    cfg->tile = 0;
    cfg->tolerance = 0.0;
    cfg->device = 0;
    return RAD_OK;
}

int rad_config_derived(const rad_config* cfg, uint32_t out[9]) {
    if (!cfg || !out) return RAD_E_INVALID;
    const uint32_t W = cfg->hemicube_side, K = cfg->hemicubes_count;
    out[0] = W;
    out[1] = W;
    out[2] = (uint32_t)(W * 2);
    out[3] = (uint32_t)(W * 1.5);
    out[4] = out[2] * out[3];
    out[5] = std::min(cfg->ocl_workitems_x, out[2]);
    out[6] = out[3] * K;
    out[7] = K;
    out[8] = out[5] ? out[2] / out[5] : 0;
    return RAD_OK;
}

int rad_create(const rad_config* cfg, rad_ctx** out) {
    if (!out) return RAD_E_INVALID;
    *out = nullptr;
    if (check_cfg(cfg) != RAD_OK) return RAD_E_INVALID;
    rad_ctx* c = new rad_ctx();
    c->cfg = *cfg;
    auto bail = [&](int code) {
        rad_destroy(c);
        return code;
    };
    if (cudaSetDevice(cfg->device) != cudaSuccess) return bail(RAD_E_CUDA);
    if (raster_init() != cudaSuccess || dense_init() != cudaSuccess) return bail(RAD_E_CUDA);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(RAD_E_CUDA);
    if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) return bail(RAD_E_CUDA);
    std::vector<BinInfo> bins;
    setup_geo(c, bins);
    if (cudaMalloc(&c->d_bins, sizeof(BinInfo) * bins.size()) != cudaSuccess) return bail(RAD_E_NOMEM);
    if (cudaMemcpy(c->d_bins, bins.data(), sizeof(BinInfo) * bins.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(RAD_E_CUDA);
    if (cudaMalloc(&c->d_fftab, sizeof(float) * c->geo.RES) != cudaSuccess) return bail(RAD_E_NOMEM);
    if (cudaMalloc(&c->d_state, sizeof(DevState)) != cudaSuccess) return bail(RAD_E_NOMEM);
    if (cudaMalloc(&c->d_aux, sizeof(DevState)) != cudaSuccess) return bail(RAD_E_NOMEM);
    if (cudaMallocHost(&c->h_flag, sizeof(uint32_t)) != cudaSuccess) return bail(RAD_E_NOMEM);
    cudaMemsetAsync(c->d_state, 0, sizeof(DevState), c->stream);
    cudaMemsetAsync(c->d_aux, 0, sizeof(DevState), c->stream);
    launch_fftab(c->geo.W, c->d_fftab, c->stream);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(RAD_E_CUDA);
    *out = c;
    return RAD_OK;
}

int rad_destroy(rad_ctx* c) {
    if (!c) return RAD_E_INVALID;
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graph(c);
    free_batch(c->shoot);
    free_batch(c->aux);
    dfree(c->d_verts);
    dfree(c->d_color);
    dfree(c->d_rho);
    dfree(c->d_rad);
    dfree(c->d_illum);
    dfree(c->d_area);
    dfree(c->d_gbox);
    dfree(c->d_nb);
    dfree(c->d_shade);
    dfree(c->d_best);
    dfree(c->d_fftab);
    dfree(c->d_bins);
    dfree(c->d_state);
    dfree(c->d_aux);
    dfree(c->d_rows);
    free_dense(c);
    if (c->h_flag) cudaFreeHost(c->h_flag);
    dfree(c->d_f3);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return RAD_OK;
}

// Host float3 array (N x 3, any host memory) -> device float4 rows, on the context's stream:
// one DMA of the caller's bytes into scratch slot `slot` of d_f3, widened on the device (no
// host-side packing loop).  A null src zeroes the rows.  Ordered in the stream, so the next
// use of the slot waits for this one.
static int upload_f3(rad_ctx* c, float4* dst, const float* src, uint32_t n, int slot) {
    if (!src) {
        RAD_CUDA(c, cudaMemsetAsync(dst, 0, sizeof(float4) * n, c->stream));
        return RAD_OK;
    }
    float* tmp = c->d_f3 + (size_t)slot * 3 * n;
    RAD_CUDA(c, cudaMemcpyAsync(tmp, src, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    launch_f3_to_f4(tmp, dst, n, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    return RAD_OK;
}

int rad_upload_scene(rad_ctx* c, const float* vertices, const int32_t* indices, const float* color,
                     const float* reflectance, const float* radiosity, const float* illumination, uint32_t n) {
    if (!c) return RAD_E_INVALID;
    if (!vertices || !color || !radiosity || !illumination || n == 0)
        return fail(c, RAD_E_INVALID, "vertices, color, radiosity and illumination are required");
    if (c->cfg.mode == RAD_MODE_PHYS && !reflectance) return fail(c, RAD_E_INVALID, "PHYS mode needs reflectance");
    if (n > 0x7FFFFFFFu) return fail(c, RAD_E_INVALID, "too many patches");
    if (indices)
        for (uint32_t i = 0; i < n; i++) {
            const int32_t b = (int32_t)(4 * i);
            const int32_t* q = indices + 6 * (size_t)i;
            if (q[0] != b || q[1] != b + 1 || q[2] != b + 2 || q[3] != b || q[4] != b + 2 || q[5] != b + 3)
                return fail(c, RAD_E_INVALID, "indices must follow the (0,1,2,0,2,3)+4i quad pattern");
        }
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    free_batch(c->shoot);
    free_batch(c->aux);
    free_dense(c);
    dfree(c->d_verts);
    dfree(c->d_color);
    dfree(c->d_rho);
    dfree(c->d_rad);
    dfree(c->d_illum);
    dfree(c->d_area);
    dfree(c->d_gbox);
    dfree(c->d_nb);
    dfree(c->d_shade);
    dfree(c->d_f3);
    c->n = n;
    c->geo.n = n;
    RAD_CUDA(c, cudaMalloc(&c->d_verts, sizeof(float) * 12 * (size_t)n));
    RAD_CUDA(c, cudaMalloc(&c->d_color, sizeof(float4) * n));
    RAD_CUDA(c, cudaMalloc(&c->d_rho, sizeof(float4) * n));
    RAD_CUDA(c, cudaMalloc(&c->d_rad, sizeof(float4) * n));
    RAD_CUDA(c, cudaMalloc(&c->d_illum, sizeof(float4) * n));
    RAD_CUDA(c, cudaMalloc(&c->d_area, sizeof(float) * n));
    RAD_CUDA(c, cudaMalloc(&c->d_gbox, sizeof(float) * 6 * (size_t)((n + 127) / 128)));
    RAD_CUDA(c, cudaMalloc(&c->d_f3, sizeof(float) * 6 * (size_t)n));
    RAD_CUDA(c, cudaMemcpyAsync(c->d_verts, vertices, sizeof(float) * 12 * (size_t)n, cudaMemcpyHostToDevice,
                                c->stream));
    int rc;
    if ((rc = upload_f3(c, c->d_color, color, n, 0))) return rc;
    if ((rc = upload_f3(c, c->d_rho, reflectance, n, 1))) return rc;
    if ((rc = upload_f3(c, c->d_rad, radiosity, n, 0))) return rc;
    if ((rc = upload_f3(c, c->d_illum, illumination, n, 1))) return rc;
    launch_areas(c->d_verts, n, c->d_area, c->stream);
    launch_group_boxes(c->d_verts, n, c->d_gbox, c->stream);
    RAD_CUDA(c, cudaMemsetAsync(c->d_state, 0, sizeof(DevState), c->stream));
    launch_power0(c->d_rad, c->d_area, n, c->d_state, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    if ((rc = alloc_batch(c, c->shoot, c->cfg.hemicubes_count, false))) return rc;
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

int rad_set_state(rad_ctx* c, const float* radiosity, const float* illumination) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    int rc;
    if (radiosity && (rc = upload_f3(c, c->d_rad, radiosity, c->n, 0))) return rc;
    if (illumination && (rc = upload_f3(c, c->d_illum, illumination, c->n, 1))) return rc;
    RAD_CUDA(c, cudaMemsetAsync(&c->d_state->stopped, 0, sizeof(uint32_t), c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

// Touches one byte per page of a pageable destination before a device-to-host copy into it.
// Where the GPU reaches host memory through the host's page tables (NVLink-C2C systems), a
// copy into never-touched pages faults each page in from the GPU side: measured on GB300,
// 155 us for a 606 KB array of fresh 64 KB pages, against ~49 us when the CPU populates them
// first.  Pinned or registered memory is left alone.  Each touched byte is written back with
// the value it holds, so the caller's array keeps its contents if the copy does not happen.
static void prefault_pageable(void* p, size_t bytes) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    if (a.type != cudaMemoryTypeUnregistered) return;
    static const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    volatile char* b = static_cast<volatile char*>(p);
    for (size_t o = 0; o < bytes; o += page) b[o] = b[o];
    if (bytes) b[bytes - 1] = b[bytes - 1];
}

// Device float4 rows -> the caller's float3 arrays: narrowed on the device into the scratch,
// then one DMA per array straight into the caller's memory.
int rad_download(rad_ctx* c, float* radiosity, float* illumination) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    const size_t n = c->n;
    float* dst[2] = {radiosity, illumination};
    const float4* src[2] = {c->d_rad, c->d_illum};
    for (int k = 0; k < 2; k++) {
        if (!dst[k]) continue;
        float* tmp = c->d_f3 + (size_t)k * 3 * n;
        prefault_pageable(dst[k], sizeof(float) * 3 * n);
        launch_f4_to_f3(src[k], tmp, c->n, c->stream);
        RAD_CUDA(c, cudaGetLastError());
        RAD_CUDA(c, cudaMemcpyAsync(dst[k], tmp, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    }
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

int rad_ff_table(rad_ctx* c, float* out, uint32_t copies) {
    if (!c || !out || copies == 0) return RAD_E_INVALID;
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    RAD_CUDA(c, cudaMemcpy(out, c->d_fftab, sizeof(float) * c->geo.RES, cudaMemcpyDeviceToHost));
    for (uint32_t k = 1; k < copies; k++) std::memcpy(out + (size_t)k * c->geo.RES, out, sizeof(float) * c->geo.RES);
    return RAD_OK;
}

int rad_select_shooters(rad_ctx* c, uint32_t* ids, uint8_t* valid) {
    if (!c || !ids || !valid) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    Batch& b = c->shoot.b;
    RAD_CUDA(c, cudaMemsetAsync(c->d_aux, 0, sizeof(DevState), c->stream));
    launch_select(c->geo, b, c->d_rad, c->d_area, c->d_aux, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    std::vector<uint32_t> v(b.K);
    RAD_CUDA(c, cudaMemcpyAsync(ids, b.shooters, sizeof(uint32_t) * b.K, cudaMemcpyDeviceToHost, c->stream));
    RAD_CUDA(c, cudaMemcpyAsync(v.data(), b.valid, sizeof(uint32_t) * b.K, cudaMemcpyDeviceToHost, c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    for (uint32_t k = 0; k < b.K; k++) valid[k] = v[k] ? 1 : 0;
    return RAD_OK;
}

int rad_render_item_buffers(rad_ctx* c, const uint32_t* shooters, uint32_t count, uint32_t* items) {
    if (!c || !items) return RAD_E_INVALID;
    int rc = run_aux(c, shooters, count, true, false);
    if (rc) return rc;
    RAD_CUDA(c, cudaMemcpy(items, c->aux.b.items, sizeof(uint32_t) * (size_t)count * c->geo.RES,
                           cudaMemcpyDeviceToHost));
    return RAD_OK;
}

int rad_reduce_item_buffers(rad_ctx* c, const uint32_t* items, uint32_t count, float* ff_rows) {
    if (!c || !items || !ff_rows || count == 0) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    int rc = alloc_batch(c, c->aux, count, true);
    if (rc) return rc;
    if ((rc = ensure_rows(c, (size_t)count * c->n))) return rc;
    Batch& b = c->aux.b;
    b.K = count;
    RAD_CUDA(c, cudaMemcpyAsync(b.items, items, sizeof(uint32_t) * (size_t)count * c->geo.RES,
                                cudaMemcpyHostToDevice, c->stream));
    RAD_CUDA(c, cudaMemsetAsync(b.Fq, 0, sizeof(unsigned long long) * (size_t)count * c->n, c->stream));
    launch_reduce_items(c->geo, b, c->d_fftab, count, c->stream);
    launch_fq_to_float(c->geo, b, count, c->d_rows, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    RAD_CUDA(c, cudaMemcpyAsync(ff_rows, c->d_rows, sizeof(float) * (size_t)count * c->n, cudaMemcpyDeviceToHost,
                                c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

int rad_ff_rows(rad_ctx* c, const uint32_t* shooters, uint32_t count, float* ff_rows) {
    if (!c || !ff_rows) return RAD_E_INVALID;
    int rc = run_aux(c, shooters, count, false, true);
    if (rc) return rc;
    if ((rc = ensure_rows(c, (size_t)count * c->n))) return rc;
    launch_fq_to_float(c->geo, c->aux.b, count, c->d_rows, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    RAD_CUDA(c, cudaMemcpyAsync(ff_rows, c->d_rows, sizeof(float) * (size_t)count * c->n, cudaMemcpyDeviceToHost,
                                c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

int rad_face_cameras(rad_ctx* c, const uint32_t* shooters, uint32_t count, float* mvp, float* frames) {
    if (!c || !mvp) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (!shooters || count == 0 || count > (uint32_t)kMaxK) return fail(c, RAD_E_INVALID, "1..1024 shooters");
    for (uint32_t i = 0; i < count; i++)
        if (shooters[i] >= c->n) return fail(c, RAD_E_INVALID, "shooter index out of range");
    int rc = alloc_batch(c, c->aux, count, false);
    if (rc) return rc;
    Batch& b = c->aux.b;
    b.K = count;
    cudaStream_t s = c->stream;
    std::vector<uint32_t> ones(count, 1u);
    RAD_CUDA(c, cudaMemsetAsync(c->d_aux, 0, sizeof(DevState), s));
    RAD_CUDA(c, cudaMemcpyAsync(b.shooters, shooters, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s));
    RAD_CUDA(c, cudaMemcpyAsync(b.valid, ones.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s));
    launch_camera(c->geo, b, c->d_verts, c->d_rad, c->d_aux, s);
    RAD_CUDA(c, cudaGetLastError());
    std::vector<float> fr((size_t)count * 8);
    RAD_CUDA(c, cudaMemcpyAsync(mvp, b.mvp, sizeof(float) * 80 * count, cudaMemcpyDeviceToHost, s));
    RAD_CUDA(c, cudaMemcpyAsync(fr.data(), b.frame, sizeof(float) * 8 * count, cudaMemcpyDeviceToHost, s));
    RAD_CUDA(c, cudaStreamSynchronize(s));
    if (frames)
        for (uint32_t i = 0; i < count; i++)
            for (int k = 0; k < 6; k++) frames[6 * i + k] = fr[8 * i + k];
    return RAD_OK;
}

int rad_shoot(rad_ctx* c, uint32_t n_shots, rad_stats* stats) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    DevState before;
    RAD_CUDA(c, cudaMemcpyAsync(&before, c->d_state, sizeof(before), cudaMemcpyDeviceToHost, c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!c->graph_exec) {
        RAD_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_batch(c);
        cudaError_t e = cudaStreamEndCapture(c->stream, &c->graph);
        if (e != cudaSuccess) return fail(c, RAD_E_CUDA, cudaGetErrorString(e));
        RAD_CUDA(c, cudaGraphInstantiate(&c->graph_exec, c->graph, 0));
    }
    RAD_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    for (uint32_t s = 0; s < n_shots; s++) {
        RAD_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream));
        if ((s & 31u) == 31u && s + 1 < n_shots) {
            RAD_CUDA(c, cudaMemcpyAsync(c->h_flag, &c->d_state->stopped, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                        c->stream));
            RAD_CUDA(c, cudaStreamSynchronize(c->stream));
            if (*c->h_flag) break;
        }
    }
    RAD_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    DevState after;
    RAD_CUDA(c, cudaMemcpyAsync(&after, c->d_state, sizeof(after), cudaMemcpyDeviceToHost, c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (stats) {
        stats->shots_done = after.shots_done - before.shots_done;
        stats->stopped = after.stopped;
        std::memcpy(stats->last_energy, after.last_energy, sizeof(float) * 3);
        stats->residual = after.residual;
        stats->hemicubes = after.hemicubes - before.hemicubes;
        stats->device_ms = ms;
    }
    if (after.overflow) return fail(c, RAD_E_OVERFLOW, "triangle or bin capacity exceeded");
    return RAD_OK;
}

// Stage-by-stage batches with events between stages (rad_profile_stages); `phases` runs the
// raster kernel that also counts SM cycles per phase (slower; rad_profile_raster_phases).
static int profile_batches(rad_ctx* c, uint32_t n_shots, double* stage_ms, rad_stats* stats, bool phases) {
    if (!c || !stage_ms) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    Batch& b = c->shoot.b;
    cudaStream_t s = c->stream;
    cudaEvent_t ev[RAD_N_STAGES + 1];
    for (auto& e : ev) RAD_CUDA(c, cudaEventCreate(&e));
    DevState before;
    RAD_CUDA(c, cudaMemcpyAsync(&before, c->d_state, sizeof(before), cudaMemcpyDeviceToHost, s));
    RAD_CUDA(c, cudaStreamSynchronize(s));
    float total_ms = 0;
    RAD_CUDA(c, cudaMemsetAsync(c->d_state->raster_counters, 0, sizeof(c->d_state->raster_counters), s));
    for (uint32_t shot = 0; shot < n_shots; shot++) {
        RAD_CUDA(c, cudaMemsetAsync(b.tri_counts, 0, sizeof(uint32_t) * b.K, s));
        RAD_CUDA(c, cudaMemsetAsync(b.bin_count, 0, sizeof(uint32_t) * (size_t)b.K * c->geo.nb, s));
        RAD_CUDA(c, cudaEventRecord(ev[0], s));
        launch_select(c->geo, b, c->d_rad, c->d_area, c->d_state, s);
        RAD_CUDA(c, cudaEventRecord(ev[1], s));
        launch_camera(c->geo, b, c->d_verts, c->d_rad, c->d_state, s);
        RAD_CUDA(c, cudaEventRecord(ev[2], s));
        launch_setup(c->geo, b, c->d_verts, c->d_gbox, c->d_state, s);
        RAD_CUDA(c, cudaEventRecord(ev[3], s));
        launch_bins(c->geo, b, c->d_state, s);
        RAD_CUDA(c, cudaEventRecord(ev[4], s));
        launch_raster(c->geo, b, c->d_fftab, c->d_state, false, true, s, true, phases);
        RAD_CUDA(c, cudaEventRecord(ev[5], s));
        launch_update(c->geo, b, c->d_color, c->d_rho, c->d_area, c->d_rad, c->d_state, s);
        RAD_CUDA(c, cudaEventRecord(ev[6], s));
        launch_emitters(c->geo, b, c->d_rad, c->d_illum, c->d_area, c->cfg.tolerance, nullptr, c->d_state, s);
        RAD_CUDA(c, cudaEventRecord(ev[7], s));
        RAD_CUDA(c, cudaGetLastError());
        RAD_CUDA(c, cudaEventSynchronize(ev[7]));
        for (int k = 0; k < RAD_N_STAGES; k++) {
            float ms = 0;
            RAD_CUDA(c, cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
            stage_ms[k] += ms;
            total_ms += ms;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    DevState after;
    RAD_CUDA(c, cudaMemcpyAsync(&after, c->d_state, sizeof(after), cudaMemcpyDeviceToHost, s));
    RAD_CUDA(c, cudaStreamSynchronize(s));
    if (stats) {
        stats->shots_done = after.shots_done - before.shots_done;
        stats->stopped = after.stopped;
        std::memcpy(stats->last_energy, after.last_energy, sizeof(float) * 3);
        stats->residual = after.residual;
        stats->hemicubes = after.hemicubes - before.hemicubes;
        stats->device_ms = total_ms;
    }
    if (after.overflow) return fail(c, RAD_E_OVERFLOW, "triangle or bin capacity exceeded");
    return RAD_OK;
}

int rad_profile_stages(rad_ctx* c, uint32_t n_shots, double* stage_ms, rad_stats* stats) {
    return profile_batches(c, n_shots, stage_ms, stats, false);
}

int rad_profile_raster_phases(rad_ctx* c, uint32_t n_shots, uint64_t* cycles, rad_stats* stats) {
    if (!c || !cycles) return RAD_E_INVALID;
    double ms[RAD_N_STAGES] = {0};
    const int rc = profile_batches(c, n_shots, ms, stats, true);
    if (rc) return rc;
    unsigned long long ctr[16];
    RAD_CUDA(c, cudaMemcpy(ctr, c->d_state->raster_counters, sizeof(ctr), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 8; k++) cycles[k] = ctr[8 + k];
    return RAD_OK;
}

// Re-derives the raster geometry for a new bin side / split / K and reallocates the
// batch buffers (the scene and the radiosity state stay on the device).
static int reconfigure(rad_ctx* c, uint32_t tile, uint32_t small, uint32_t K) {
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    drop_graph(c);
    free_batch(c->shoot);
    free_batch(c->aux);
    c->cfg.tile = tile;
    c->cfg.small_tri_pixels = small;
    c->cfg.hemicubes_count = K;
    const uint32_t n = c->geo.n;
    std::vector<BinInfo> bins;
    setup_geo(c, bins);
    c->geo.n = n;
    dfree(c->d_bins);
    RAD_CUDA(c, cudaMalloc(&c->d_bins, sizeof(BinInfo) * bins.size()));
    RAD_CUDA(c, cudaMemcpy(c->d_bins, bins.data(), sizeof(BinInfo) * bins.size(), cudaMemcpyHostToDevice));
    return alloc_batch(c, c->shoot, K, false);
}

// Device time of render + reduce of `count` shooters with the aux batch (best of reps).
static int time_pipeline(rad_ctx* c, const std::vector<uint32_t>& sh, int reps, float* best_ms) {
    const uint32_t count = (uint32_t)sh.size();
    int rc = alloc_batch(c, c->aux, count, false);
    if (rc) return rc;
    Batch& b = c->aux.b;
    b.K = count;
    cudaStream_t s = c->stream;
    std::vector<uint32_t> ones(count, 1u);
    RAD_CUDA(c, cudaMemcpyAsync(b.shooters, sh.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s));
    RAD_CUDA(c, cudaMemcpyAsync(b.valid, ones.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s));
    *best_ms = 1e30f;
    for (int r = 0; r < reps + 1; r++) {
        RAD_CUDA(c, cudaMemsetAsync(c->d_aux, 0, sizeof(DevState), s));
        RAD_CUDA(c, cudaMemsetAsync(b.tri_counts, 0, sizeof(uint32_t) * count, s));
        RAD_CUDA(c, cudaMemsetAsync(b.bin_count, 0, sizeof(uint32_t) * (size_t)count * c->geo.nb, s));
        RAD_CUDA(c, cudaEventRecord(c->ev0, s));
        launch_camera(c->geo, b, c->d_verts, c->d_rad, c->d_aux, s);
        launch_setup(c->geo, b, c->d_verts, c->d_gbox, c->d_aux, s);
        launch_bins(c->geo, b, c->d_aux, s);
        launch_raster(c->geo, b, c->d_fftab, c->d_aux, false, true, s);
        RAD_CUDA(c, cudaEventRecord(c->ev1, s));
        RAD_CUDA(c, cudaMemsetAsync(b.Fq, 0, sizeof(unsigned long long) * (size_t)count * c->n, s));
        RAD_CUDA(c, cudaGetLastError());
        RAD_CUDA(c, cudaEventSynchronize(c->ev1));
        float ms = 0;
        RAD_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        if (r > 0 && ms < *best_ms) *best_ms = ms;  // first pass warms up
    }
    DevState st;
    RAD_CUDA(c, cudaMemcpy(&st, c->d_aux, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.overflow) *best_ms = 1e30f;
    return RAD_OK;
}

int rad_autotune(rad_ctx* c, uint32_t flags, rad_tuning* out) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    // sample shooters: the current top K (or an even spread when nothing has energy)
    const uint32_t K0 = c->cfg.hemicubes_count;
    std::vector<uint32_t> ids(K0);
    std::vector<uint8_t> valid(K0);
    int rc = rad_select_shooters(c, ids.data(), valid.data());
    if (rc) return rc;
    std::vector<uint32_t> sh;
    for (uint32_t k = 0; k < K0; k++)
        if (valid[k]) sh.push_back(ids[k]);
    const uint32_t want = std::max<uint32_t>(8, std::min<uint32_t>(K0, 64));
    for (uint32_t i = 0; sh.size() < want && i < want; i++) sh.push_back((uint32_t)(((uint64_t)i * 2654435761u) % c->n));
    const uint32_t tiles[3] = {16, 32, 64};
    const uint32_t smalls[4] = {64, 256, 1024, 4096};
    uint32_t best_t = 0, best_s = 0, cand = 0;
    float best = 1e30f;
    for (uint32_t t : tiles) {
        if (t > c->geo.W) continue;
        for (uint32_t sm : smalls) {
            if ((rc = reconfigure(c, t, sm, K0))) return rc;
            float ms;
            if ((rc = time_pipeline(c, sh, 2, &ms))) return rc;
            cand++;
            if (ms < best) {
                best = ms;
                best_t = t;
                best_s = sm;
            }
        }
    }
    if (best_t == 0) return fail(c, RAD_E_OVERFLOW, "no raster configuration fit the capacities");
    uint32_t best_k = K0;
    if (flags & RAD_TUNE_K) {
        // throughput of the whole batch at K; the smallest K within 10% of the best rate wins
        const uint32_t ks[5] = {8, 16, 32, 64, 128};
        double rate[5] = {0, 0, 0, 0, 0}, top = 0;
        for (int i = 0; i < 5; i++) {
            if ((rc = reconfigure(c, best_t, best_s, ks[i]))) return rc;
            std::vector<uint32_t> shk;
            for (uint32_t k = 0; k < ks[i]; k++) shk.push_back(sh[k % sh.size()]);
            float ms;
            if ((rc = time_pipeline(c, shk, 2, &ms))) return rc;
            rate[i] = ks[i] / (double)ms;
            top = std::max(top, rate[i]);
            cand++;
        }
        for (int i = 0; i < 5; i++)
            if (rate[i] >= 0.9 * top) {
                best_k = ks[i];
                break;
            }
    }
    if ((rc = reconfigure(c, best_t, best_s, best_k))) return rc;
    if (out) {
        out->tile = best_t;
        out->small_tri_pixels = best_s;
        out->hemicubes_count = best_k;
        out->candidates = cand;
        out->us_per_hemicube = 1000.0 * best / (double)sh.size();
    }
    return RAD_OK;
}

// Every form-factor row, 128 shooters per chunk, queued back to back on the context's
// stream: the chunk's shooter ids are a slice of one device array of 0..n-1, the row
// conversion zeroes the exact sums it has read (so the next chunk starts from zero), and
// the capacity flags are read once at the end.
}  // extern "C"

uint32_t ctx_dense_chunk(const rad_ctx* c) { return std::min<uint32_t>(128, c->n); }

int ctx_dense_alloc(rad_ctx* c, bool fp32, bool shoot) {
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    const uint32_t n = c->n, ld = (n + 63u) & ~63u;
    free_dense(c);
    c->dense_ld = ld;
    c->dense_shoot = shoot;
    RAD_CUDA(c, cudaMalloc(&c->d_F16, sizeof(__nv_bfloat16) * (size_t)n * ld));
    RAD_CUDA(c, cudaMalloc(&c->d_scale, sizeof(float) * n));
    if (fp32) RAD_CUDA(c, cudaMalloc(&c->d_F32, sizeof(float) * (size_t)n * ld));
    if (shoot) {
        RAD_CUDA(c, cudaMalloc(&c->d_F16T, sizeof(__nv_bfloat16) * (size_t)n * ld));
        if (fp32) RAD_CUDA(c, cudaMalloc(&c->d_F32T, sizeof(float) * (size_t)n * ld));
        RAD_CUDA(c, cudaMalloc(&c->d_inv_area, sizeof(float) * n));
        RAD_CUDA(c, cudaMalloc(&c->d_wT, sizeof(float) * n));
    }
    const uint32_t chunk = ctx_dense_chunk(c);
    int rc = alloc_batch(c, c->aux, chunk, false);
    if (rc) return rc;
    std::vector<uint32_t> ones(chunk, 1u);
    Batch& b = c->aux.b;
    RAD_CUDA(c, cudaMemcpyAsync(b.valid, ones.data(), sizeof(uint32_t) * chunk, cudaMemcpyHostToDevice, c->stream));
    RAD_CUDA(c, cudaMemsetAsync(b.Fq, 0, sizeof(unsigned long long) * (size_t)chunk * n, c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

// One hemicube per patch, `chunk` at a time: camera, setup, bins, raster with the fused
// exact reduction, then k_dense_rows turns the chunk's exact sums into FP32 / BF16 rows and
// clears them for the next chunk.
void ctx_enqueue_dense_capture(rad_ctx* c, const uint32_t* d_ids, cudaStream_t s) {
    const uint32_t n = c->n, chunk = ctx_dense_chunk(c);
    Batch b = c->aux.b;
    cudaMemsetAsync(c->d_aux, 0, sizeof(DevState), s);
    for (uint32_t first = 0; first < n; first += chunk) {
        const uint32_t cnt = std::min(chunk, n - first);
        b.K = cnt;
        b.shooters = const_cast<uint32_t*>(d_ids) + first;
        cudaMemsetAsync(b.tri_counts, 0, sizeof(uint32_t) * cnt, s);
        cudaMemsetAsync(b.bin_count, 0, sizeof(uint32_t) * (size_t)cnt * c->geo.nb, s);
        launch_camera(c->geo, b, c->d_verts, c->d_rad, c->d_aux, s);
        launch_setup(c->geo, b, c->d_verts, c->d_gbox, c->d_aux, s);
        launch_bins(c->geo, b, c->d_aux, s);
        launch_raster(c->geo, b, c->d_fftab, c->d_aux, false, true, s);
        launch_dense_rows(b.Fq, cnt, n, c->dense_ld, first, c->d_F32, c->d_F16, c->d_scale, s);
    }
    if (c->dense_shoot)
        launch_shoot_form(n, c->dense_ld, c->d_F32, c->d_F32T, c->d_F16, c->d_F16T, c->d_area, c->d_scale,
                          c->d_inv_area, c->d_wT, s);
}

void ctx_dense_resid(const rad_ctx* c, const float* X, const float* E, uint32_t R, float* r, double* nrm,
                     float* scratch, uint32_t* err, cudaStream_t s) {
    if (c->dense_shoot)
        launch_sgemm_resid(c->d_F32T, c->n, c->dense_ld, X, E, c->d_rho, R, r, nrm, scratch, err, s, c->d_area,
                           c->d_inv_area);
    else
        launch_sgemm_resid(c->d_F32, c->n, c->dense_ld, X, E, c->d_rho, R, r, nrm, scratch, err, s);
}

void ctx_dense_pack(const rad_ctx* c, const float* X, uint32_t R, __nv_bfloat16* Xt, uint32_t Rpad,
                    cudaStream_t s) {
    launch_pack_bf16(X, c->n, R, c->dense_ld, Xt, Rpad, s, c->dense_shoot ? c->d_wT : nullptr);
}

// Gather form: the rows are F_ij / s_i, so the sweep multiplies by s_i.  Shoot form: the
// transposed rows are F_ji / s_j and the right-hand side carries s_j A_j, so the sweep
// divides by A_i and the BF16 copy of the update is multiplied by s_i A_i for the next sweep.
const __nv_bfloat16* ctx_dense_sweep(const rad_ctx* c, TcEpilogue& ep) {
    ep.rho = c->d_rho;
    if (c->dense_shoot) {
        ep.scale = c->d_inv_area;
        ep.wscale = c->d_wT;
        return c->d_F16T;
    }
    ep.scale = c->d_scale;
    ep.wscale = nullptr;
    return c->d_F16;
}

extern "C" {

int rad_dense_capture(rad_ctx* c, uint32_t flags, double* device_ms) {
    if (!c) return RAD_E_INVALID;
    if (flags & ~(RAD_DENSE_FP32 | RAD_DENSE_SHOOT_FORM)) return fail(c, RAD_E_INVALID, "unknown capture flags");
    if ((flags & RAD_DENSE_SHOOT_FORM) && c->cfg.mode != RAD_MODE_PHYS)
        return fail(c, RAD_E_STATE, "the shoot form needs PHYS areas");
    int rc = ctx_dense_alloc(c, (flags & RAD_DENSE_FP32) != 0, (flags & RAD_DENSE_SHOOT_FORM) != 0);
    if (rc) return rc;
    const uint32_t n = c->n;
    cudaStream_t s = c->stream;
    uint32_t* d_ids = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto done = [&](int code) {
        if (d_ids) cudaFree(d_ids);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return code;
    };
    std::vector<uint32_t> ids(n);
    for (uint32_t i = 0; i < n; i++) ids[i] = i;
    if (cudaMalloc(&d_ids, sizeof(uint32_t) * n) != cudaSuccess) return done(fail(c, RAD_E_NOMEM, "cudaMalloc ids"));
    bool ok = cudaMemcpyAsync(d_ids, ids.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess &&
              cudaEventRecord(e0, s) == cudaSuccess;
    if (ok) {
        ctx_enqueue_dense_capture(c, d_ids, s);
        ok = cudaGetLastError() == cudaSuccess;
    }
    ok = ok && cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
    if (!ok) return done(fail(c, RAD_E_CUDA, "dense capture: CUDA error"));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    DevState st;
    if (cudaMemcpy(&st, c->d_aux, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess)
        return done(fail(c, RAD_E_CUDA, "dense capture: state read"));
    if (st.overflow) return done(fail(c, RAD_E_OVERFLOW, "triangle or bin capacity exceeded"));
    if (device_ms) *device_ms = ms;
    c->dense_ready = true;
    return done(RAD_OK);
}

int rad_dense_rows(rad_ctx* c, uint32_t first, uint32_t count, float* f32, uint16_t* bf16, float* scale) {
    if (!c) return RAD_E_INVALID;
    if (!c->dense_ready) return fail(c, RAD_E_STATE, "no dense capture");
    if ((uint64_t)first + count > c->n) return fail(c, RAD_E_INVALID, "rows out of range");
    const size_t n = c->n, ld = c->dense_ld;
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    if (f32) {
        if (!c->d_F32) return fail(c, RAD_E_STATE, "FP32 rows were not kept");
        RAD_CUDA(c, cudaMemcpy2D(f32, n * 4, c->d_F32 + (size_t)first * ld, ld * 4, n * 4, count, cudaMemcpyDeviceToHost));
    }
    if (bf16)
        RAD_CUDA(c, cudaMemcpy2D(bf16, n * 2, c->d_F16 + (size_t)first * ld, ld * 2, n * 2, count, cudaMemcpyDeviceToHost));
    if (scale) RAD_CUDA(c, cudaMemcpy(scale, c->d_scale + first, 4 * (size_t)count, cudaMemcpyDeviceToHost));
    return RAD_OK;
}

int rad_gather_solve(rad_ctx* c, const float* emission, uint32_t R, const float* guess, double tol, uint32_t max_outer,
                     uint32_t sweeps, float* radiosity, rad_gather_stats* stats) {
    if (!c || !emission || !radiosity || R == 0) return RAD_E_INVALID;
    if (!c->dense_ready || !c->d_F32) return fail(c, RAD_E_STATE, "needs rad_dense_capture with RAD_DENSE_FP32");
    if (c->cfg.mode != RAD_MODE_PHYS) return fail(c, RAD_E_STATE, "the gathering solve needs PHYS reflectance");
    const uint32_t Rpad = gemm_tc_width(R);
    if (!Rpad) return fail(c, RAD_E_INVALID, "at most 256 right-hand sides");
    const uint32_t n = c->n, ld = c->dense_ld;
    const size_t nr = (size_t)n * R;
    cudaStream_t s = c->stream;
    float *dE = nullptr, *dB = nullptr, *dr = nullptr, *dd = nullptr, *dpart = nullptr, *dxp = nullptr;
    __nv_bfloat16* d16[2] = {nullptr, nullptr};
    const uint32_t ksplit = gemm_tc_ksplit(n, ld, Rpad);
    double* dnrm = nullptr;
    uint32_t* derr = nullptr;
    int rc = RAD_OK;
    auto cleanup = [&]() {
        cudaFree(dE); cudaFree(dB); cudaFree(dr); cudaFree(dd);
        cudaFree(d16[0]); cudaFree(d16[1]); cudaFree(dnrm); cudaFree(derr); cudaFree(dpart); cudaFree(dxp);
    };
#define G_CUDA(call)                                                                                  \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            c->err = std::string(#call) + ": " + cudaGetErrorString(e_);                              \
            cleanup();                                                                                \
            return e_ == cudaErrorMemoryAllocation ? RAD_E_NOMEM : RAD_E_CUDA;                        \
        }                                                                                             \
    } while (0)
    G_CUDA(cudaMalloc(&dE, 4 * nr));
    G_CUDA(cudaMalloc(&dB, 4 * nr));
    G_CUDA(cudaMalloc(&dr, 4 * nr));
    G_CUDA(cudaMalloc(&dd, 4 * nr));
    G_CUDA(cudaMalloc(&d16[0], 2 * (size_t)Rpad * ld));
    G_CUDA(cudaMalloc(&d16[1], 2 * (size_t)Rpad * ld));
    // The sweeps' epilogue writes only columns c < R and rows i < n of its BF16 output, and
    // the next sweep multiplies the whole padded operand by F's zero padding: the padding
    // must hold zeros, not leftover bits (0 x NaN = NaN).  k_pack_bf16 rewrites d16[0] in
    // full; d16[1] is cleared once here.
    G_CUDA(cudaMemsetAsync(d16[0], 0, 2 * (size_t)Rpad * ld, s));
    G_CUDA(cudaMemsetAsync(d16[1], 0, 2 * (size_t)Rpad * ld, s));
    G_CUDA(cudaMalloc(&dnrm, 8 * (size_t)R));
    if (const size_t xs = sgemm_resid_scratch_floats(R, ld)) G_CUDA(cudaMalloc(&dxp, 4 * xs));
    if (ksplit > 1) G_CUDA(cudaMalloc(&dpart, 4 * nr * ksplit));
    G_CUDA(cudaMalloc(&derr, 4));
    G_CUDA(cudaMemsetAsync(derr, 0, 4, s));
    G_CUDA(cudaMemcpyAsync(dE, emission, 4 * nr, cudaMemcpyHostToDevice, s));
    G_CUDA(cudaMemcpyAsync(dB, guess ? guess : emission, 4 * nr, cudaMemcpyHostToDevice, s));
    std::vector<double> enorm(R, 0.0), nrm(R);
    for (uint32_t col = 0; col < R; col++) {
        double a = 0;
        for (uint32_t i = 0; i < n; i++) a += (double)emission[(size_t)col * n + i] * emission[(size_t)col * n + i];
        enorm[col] = std::sqrt(a);
    }
    bool finite = true;
    for (uint32_t col = 0; col < R; col++) finite = finite && std::isfinite(enorm[col]);
    for (size_t i = 0; guess && finite && i < nr; i++) finite = std::isfinite(guess[i]);
    if (!finite) {
        cleanup();
        return fail(c, RAD_E_INVALID, "emission or guess holds NaN / inf");
    }
    cudaEvent_t ev[4];
    for (auto& e : ev) G_CUDA(cudaEventCreate(&e));
    G_CUDA(cudaEventRecord(ev[0], s));
    rad_gather_stats st{};
    double sweep_ms = 0, resid_ms = 0;
    for (uint32_t outer = 0;; outer++) {
        G_CUDA(cudaMemsetAsync(dnrm, 0, 8 * (size_t)R, s));
        G_CUDA(cudaEventRecord(ev[2], s));
        ctx_dense_resid(c, dB, dE, R, dr, dnrm, dxp, derr, s);
        G_CUDA(cudaEventRecord(ev[3], s));
        G_CUDA(cudaGetLastError());
        G_CUDA(cudaMemcpyAsync(nrm.data(), dnrm, 8 * (size_t)R, cudaMemcpyDeviceToHost, s));
        G_CUDA(cudaStreamSynchronize(s));
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[2], ev[3]);
        resid_ms += ms;
        double res = 0;
        bool bad = false;
        for (uint32_t col = 0; col < R; col++) {
            bad = bad || !std::isfinite(nrm[col]);
            if (enorm[col] > 0) res = std::max(res, std::sqrt(nrm[col]) / enorm[col]);
        }
        st.outer = outer + 1;
        if (outer == 0) st.initial_residual = bad ? NAN : res;
        st.residual = bad ? NAN : res;
        if (bad) {  // NaN would compare as converged
            rc = fail(c, RAD_E_NUMERIC, "a residual norm is not finite");
            break;
        }
        if (res <= tol || outer >= max_outer) break;
        // correction: d = r + rho o (F16 d), d0 = r
        if (sweeps == 0) {
            G_CUDA(cudaMemcpyAsync(dd, dr, 4 * nr, cudaMemcpyDeviceToDevice, s));
        } else {
            ctx_dense_pack(c, dr, R, d16[0], Rpad, s);
            G_CUDA(cudaEventRecord(ev[2], s));
            int cur = 0;
            for (uint32_t k = 0; k < sweeps; k++) {
                TcEpilogue ep{};
                const __nv_bfloat16* M = ctx_dense_sweep(c, ep);
                ep.mode = 1;
                ep.n = n;
                ep.R = R;
                ep.resid = dr;
                ep.out = dd;
                ep.out16 = d16[cur ^ 1];
                ep.ld16 = ld;
                ep.err = derr;
                ep.partial = dpart;
                ep.ksplit = ksplit;
                if (launch_gemm_tc(M, n, ld, d16[cur], Rpad, ep, s) != 0) {
                    cleanup();
                    return fail(c, RAD_E_CUDA, "tcgen05 GEMM launch failed");
                }
                cur ^= 1;
                st.sweeps++;
            }
            G_CUDA(cudaEventRecord(ev[3], s));
            G_CUDA(cudaEventSynchronize(ev[3]));
            ms = 0;
            cudaEventElapsedTime(&ms, ev[2], ev[3]);
            sweep_ms += ms;
        }
        launch_axpy(dB, dd, nr, s);
        G_CUDA(cudaGetLastError());
    }
    G_CUDA(cudaEventRecord(ev[1], s));
    G_CUDA(cudaEventSynchronize(ev[1]));
    float total = 0;
    cudaEventElapsedTime(&total, ev[0], ev[1]);
    for (auto& e : ev) cudaEventDestroy(e);
    uint32_t herr = 0;
    G_CUDA(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
    G_CUDA(cudaMemcpy(radiosity, dB, 4 * nr, cudaMemcpyDeviceToHost));
#undef G_CUDA
    cleanup();
    st.device_ms = total;
    st.sweep_ms = sweep_ms;
    st.resid_ms = resid_ms;
    if (stats) *stats = st;
    if (herr) rc = fail(c, RAD_E_TIMEOUT, "a tcgen05 or residual pipeline wait timed out");
    return rc;
}

int rad_gather_residual(rad_ctx* c, const float* emission, uint32_t R, const float* radiosity, float* residual) {
    if (!c || !emission || !radiosity || !residual || R == 0) return RAD_E_INVALID;
    if (!c->dense_ready || !c->d_F32) return fail(c, RAD_E_STATE, "needs rad_dense_capture with RAD_DENSE_FP32");
    const size_t nr = (size_t)c->n * R;
    float *dE = nullptr, *dB = nullptr, *dr = nullptr, *dxp = nullptr;
    uint32_t* derr = nullptr;
    uint32_t herr = 0;
    int rc = RAD_OK;
    const size_t xs = sgemm_resid_scratch_floats(R, c->dense_ld);
    if (cudaMalloc(&dE, 4 * nr) != cudaSuccess || cudaMalloc(&dB, 4 * nr) != cudaSuccess ||
        cudaMalloc(&dr, 4 * nr) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess ||
        (xs && cudaMalloc(&dxp, 4 * xs) != cudaSuccess))
        rc = fail(c, RAD_E_NOMEM, "residual buffers");
    if (!rc) {
        cudaMemsetAsync(derr, 0, 4, c->stream);
        cudaMemcpyAsync(dE, emission, 4 * nr, cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(dB, radiosity, 4 * nr, cudaMemcpyHostToDevice, c->stream);
        ctx_dense_resid(c, dB, dE, R, dr, nullptr, dxp, derr, c->stream);
        cudaMemcpyAsync(residual, dr, 4 * nr, cudaMemcpyDeviceToHost, c->stream);
        cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, c->stream);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
            rc = fail(c, RAD_E_CUDA, "residual GEMM failed");
        else if (herr)
            rc = fail(c, RAD_E_TIMEOUT, "a residual pipeline wait timed out");
    }
    cudaFree(dE);
    cudaFree(dB);
    cudaFree(dr);
    cudaFree(dxp);
    cudaFree(derr);
    return rc;
}

int rad_shoot_residual(rad_ctx* c, const float* emission, uint32_t R, const float* radiosity, float* residual) {
    if (!c || !emission || !radiosity || !residual || R == 0) return RAD_E_INVALID;
    if (!c->dense_ready || !c->d_F32) return fail(c, RAD_E_STATE, "needs rad_dense_capture with RAD_DENSE_FP32");
    const size_t nr = (size_t)c->n * R;
    float *dE = nullptr, *dB = nullptr, *dr = nullptr;
    double* dacc = nullptr;
    int rc = RAD_OK;
    if (cudaMalloc(&dE, 4 * nr) != cudaSuccess || cudaMalloc(&dB, 4 * nr) != cudaSuccess ||
        cudaMalloc(&dr, 4 * nr) != cudaSuccess || cudaMalloc(&dacc, 8 * nr) != cudaSuccess)
        rc = fail(c, RAD_E_NOMEM, "residual buffers");
    if (!rc) {
        cudaMemcpyAsync(dE, emission, 4 * nr, cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(dB, radiosity, 4 * nr, cudaMemcpyHostToDevice, c->stream);
        launch_shoot_resid(c->d_F32, c->n, c->dense_ld, dB, dE, c->d_rho, c->d_area, R, dacc, dr, c->stream);
        cudaMemcpyAsync(residual, dr, 4 * nr, cudaMemcpyDeviceToHost, c->stream);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
            rc = fail(c, RAD_E_CUDA, "shooting-form residual failed");
    }
    cudaFree(dE);
    cudaFree(dB);
    cudaFree(dr);
    cudaFree(dacc);
    return rc;
}

int rad_selftest_bounded_wait(int device, uint32_t limit_us, double* waited_ms) {
    if (limit_us == 0 || limit_us > 2000000u) return RAD_E_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return RAD_E_CUDA;
    uint32_t* derr = nullptr;
    if (cudaMalloc(&derr, 4) != cudaSuccess) return RAD_E_NOMEM;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = RAD_OK;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        rc = RAD_E_CUDA;
    uint32_t herr = 0;
    if (!rc) {
        cudaMemsetAsync(derr, 0, 4, s);
        cudaEventRecord(e0, s);
        if (launch_wait_selftest(derr, 1000ull * limit_us, s) != 0) rc = RAD_E_CUDA;
        cudaEventRecord(e1, s);
        cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = RAD_E_CUDA;
    }
    if (!rc) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (waited_ms) *waited_ms = ms;
        rc = herr ? RAD_E_TIMEOUT : RAD_OK;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(derr);
    return rc;
}

int rad_bf16_gemm(int device, const uint16_t* A, const uint16_t* Bt, uint32_t n, uint32_t k, uint32_t R, float* C) {
    if (!A || !Bt || !C || n == 0 || k == 0 || R == 0) return RAD_E_INVALID;
    const uint32_t Rpad = gemm_tc_width(R);
    if (!Rpad) return RAD_E_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return RAD_E_CUDA;
    const uint32_t ld = (k + 63u) & ~63u;
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    float *dC = nullptr, *dpart = nullptr;
    uint32_t* derr = nullptr;
    int rc = RAD_OK;
    // the gathering solve's split-K policy, so that the split path and its finalize run too
    const uint32_t ksplit = gemm_tc_ksplit(n, ld, Rpad);
    if (cudaMalloc(&dA, 2 * (size_t)n * ld) != cudaSuccess || cudaMalloc(&dB, 2 * (size_t)Rpad * ld) != cudaSuccess ||
        cudaMalloc(&dC, 4 * (size_t)n * R) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess ||
        (ksplit > 1 && cudaMalloc(&dpart, 4 * (size_t)n * R * ksplit) != cudaSuccess))
        rc = RAD_E_NOMEM;
    if (!rc) {
        cudaMemset(dA, 0, 2 * (size_t)n * ld);
        cudaMemset(dB, 0, 2 * (size_t)Rpad * ld);
        cudaMemset(derr, 0, 4);
        cudaMemcpy2D(dA, 2 * ld, A, 2 * (size_t)k, 2 * (size_t)k, n, cudaMemcpyHostToDevice);
        cudaMemcpy2D(dB, 2 * ld, Bt, 2 * (size_t)k, 2 * (size_t)k, R, cudaMemcpyHostToDevice);
        TcEpilogue ep{};
        ep.mode = 0;
        ep.n = n;
        ep.R = R;
        ep.out = dC;
        ep.err = derr;
        ep.partial = dpart;
        ep.ksplit = ksplit;
        if (launch_gemm_tc(dA, n, ld, dB, Rpad, ep, 0) != 0) rc = RAD_E_CUDA;
        if (!rc && cudaDeviceSynchronize() != cudaSuccess) rc = RAD_E_CUDA;
        uint32_t herr = 0;
        if (!rc) cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
        if (!rc && herr) rc = RAD_E_TIMEOUT;
        if (!rc) cudaMemcpy(C, dC, 4 * (size_t)n * R, cudaMemcpyDeviceToHost);
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(derr);
    cudaFree(dpart);
    return rc;
}

namespace {
__global__ void k_gather_flags(DevState* const* states, uint32_t count, uint32_t* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = states[i]->stopped;
}
}  // namespace

struct rad_multi {
    std::vector<rad_ctx*> ctxs;
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> fork, join;
    DevState** d_states = nullptr;
    uint32_t* d_flags = nullptr;
    uint32_t* h_flags = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
};

int rad_multi_destroy(rad_multi* m) {
    if (!m) return RAD_E_INVALID;
    if (m->stream) cudaStreamSynchronize(m->stream);
    if (m->exec) cudaGraphExecDestroy(m->exec);
    if (m->graph) cudaGraphDestroy(m->graph);
    for (auto e : m->fork) cudaEventDestroy(e);
    for (auto e : m->join) cudaEventDestroy(e);
    if (m->t0) cudaEventDestroy(m->t0);
    if (m->t1) cudaEventDestroy(m->t1);
    cudaFree(m->d_states);
    cudaFree(m->d_flags);
    if (m->h_flags) cudaFreeHost(m->h_flags);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return RAD_OK;
}

int rad_multi_create(rad_ctx* const* ctxs, uint32_t count, rad_multi** out) {
    if (!ctxs || count == 0 || !out) return RAD_E_INVALID;
    *out = nullptr;
    const int dev = ctxs[0]->cfg.device;
    for (uint32_t i = 0; i < count; i++)
        if (!ctxs[i] || !ctxs[i]->n || ctxs[i]->cfg.device != dev) return RAD_E_INVALID;
    if (cudaSetDevice(dev) != cudaSuccess) return RAD_E_CUDA;
    rad_multi* m = new rad_multi();
    m->ctxs.assign(ctxs, ctxs + count);
    auto bail = [&](int code) {
        rad_multi_destroy(m);
        return code;
    };
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(RAD_E_CUDA);
    if (cudaEventCreate(&m->t0) != cudaSuccess || cudaEventCreate(&m->t1) != cudaSuccess) return bail(RAD_E_CUDA);
    m->fork.resize(count);
    m->join.resize(count);
    for (uint32_t i = 0; i < count; i++) {
        if (cudaEventCreateWithFlags(&m->fork[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&m->join[i], cudaEventDisableTiming) != cudaSuccess)
            return bail(RAD_E_CUDA);
        cudaStreamSynchronize(ctxs[i]->stream);
    }
    std::vector<DevState*> st(count);
    for (uint32_t i = 0; i < count; i++) st[i] = ctxs[i]->d_state;
    if (cudaMalloc(&m->d_states, sizeof(DevState*) * count) != cudaSuccess ||
        cudaMalloc(&m->d_flags, sizeof(uint32_t) * count) != cudaSuccess ||
        cudaMallocHost(&m->h_flags, sizeof(uint32_t) * count) != cudaSuccess)
        return bail(RAD_E_NOMEM);
    cudaMemcpy(m->d_states, st.data(), sizeof(DevState*) * count, cudaMemcpyHostToDevice);
    if (cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return bail(RAD_E_CUDA);
    for (uint32_t i = 0; i < count; i++) {
        cudaEventRecord(m->fork[i], m->stream);
        cudaStreamWaitEvent(ctxs[i]->stream, m->fork[i], 0);
        enqueue_batch(ctxs[i]);
        cudaEventRecord(m->join[i], ctxs[i]->stream);
        cudaStreamWaitEvent(m->stream, m->join[i], 0);
    }
    k_gather_flags<<<(count + 255) / 256, 256, 0, m->stream>>>(m->d_states, count, m->d_flags);
    cudaMemcpyAsync(m->h_flags, m->d_flags, sizeof(uint32_t) * count, cudaMemcpyDeviceToHost, m->stream);
    if (cudaStreamEndCapture(m->stream, &m->graph) != cudaSuccess) return bail(RAD_E_CUDA);
    if (cudaGraphInstantiate(&m->exec, m->graph, 0) != cudaSuccess) return bail(RAD_E_CUDA);
    *out = m;
    return RAD_OK;
}

int rad_multi_shoot(rad_multi* m, uint32_t n_replays, uint32_t* stop_replay, double* stop_ms, uint32_t* replays,
                    double* device_ms) {
    if (!m) return RAD_E_INVALID;
    const uint32_t count = (uint32_t)m->ctxs.size();
    std::vector<uint32_t> at(count, 0);
    std::vector<double> at_ms(count, 0.0);
    double total = 0;
    uint32_t done_replays = 0;
    for (uint32_t r = 0; r < n_replays; r++) {
        if (cudaEventRecord(m->t0, m->stream) != cudaSuccess) return RAD_E_CUDA;
        if (cudaGraphLaunch(m->exec, m->stream) != cudaSuccess) return RAD_E_CUDA;
        if (cudaEventRecord(m->t1, m->stream) != cudaSuccess) return RAD_E_CUDA;
        if (cudaStreamSynchronize(m->stream) != cudaSuccess) return RAD_E_CUDA;
        float ms = 0;
        cudaEventElapsedTime(&ms, m->t0, m->t1);
        total += ms;
        done_replays = r + 1;
        uint32_t open = 0;
        for (uint32_t i = 0; i < count; i++) {
            if (m->h_flags[i] && !at[i]) {
                at[i] = r + 1;
                at_ms[i] = total;
            }
            open += at[i] == 0;
        }
        if (!open) break;
    }
    for (uint32_t i = 0; i < count; i++) {
        DevState s;
        cudaMemcpy(&s, m->ctxs[i]->d_state, sizeof(s), cudaMemcpyDeviceToHost);
        if (s.overflow) return RAD_E_OVERFLOW;
    }
    if (stop_replay) std::memcpy(stop_replay, at.data(), sizeof(uint32_t) * count);
    if (stop_ms) std::memcpy(stop_ms, at_ms.data(), sizeof(double) * count);
    if (replays) *replays = done_replays;
    if (device_ms) *device_ms = total;
    return RAD_OK;
}

int rad_upload_neighbours(rad_ctx* c, const uint32_t* neighbours) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (!neighbours) return fail(c, RAD_E_INVALID, "neighbours are required");
    for (size_t i = 0; i < (size_t)c->n * 8; i++)
        if (neighbours[i] >= c->n) return fail(c, RAD_E_INVALID, "neighbour index out of range");
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!c->d_nb) RAD_CUDA(c, cudaMalloc(&c->d_nb, sizeof(uint32_t) * 8 * (size_t)c->n));
    RAD_CUDA(c, cudaMemcpy(c->d_nb, neighbours, sizeof(uint32_t) * 8 * (size_t)c->n, cudaMemcpyHostToDevice));
    return RAD_OK;
}

int rad_display_colors_device(rad_ctx* c, float* d_colors, float* d_radiative) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (d_colors && !c->d_nb) return fail(c, RAD_E_STATE, "no neighbours uploaded");
    if (!d_colors && !d_radiative) return RAD_OK;
    launch_shade(c->n, c->d_nb, c->d_color, c->d_rad, c->d_illum, d_colors, d_radiative, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAD_OK;
}

int rad_display_colors(rad_ctx* c, float* colors, float* radiative) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (colors && !c->d_nb) return fail(c, RAD_E_STATE, "no neighbours uploaded");
    if (!colors && !radiative) return RAD_OK;
    const size_t per = 12 * (size_t)c->n;
    if (!c->d_shade) RAD_CUDA(c, cudaMalloc(&c->d_shade, sizeof(float) * 2 * per));
    int rc = rad_display_colors_device(c, colors ? c->d_shade : nullptr, radiative ? c->d_shade + per : nullptr);
    if (rc) return rc;
    if (colors) RAD_CUDA(c, cudaMemcpy(colors, c->d_shade, sizeof(float) * per, cudaMemcpyDeviceToHost));
    if (radiative) RAD_CUDA(c, cudaMemcpy(radiative, c->d_shade + per, sizeof(float) * per, cudaMemcpyDeviceToHost));
    return RAD_OK;
}

int rad_highest_patch(rad_ctx* c, uint32_t* id) {
    if (!c || !id) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (!c->d_best) RAD_CUDA(c, cudaMalloc(&c->d_best, sizeof(unsigned long long)));
    RAD_CUDA(c, cudaMemsetAsync(c->d_best, 0, sizeof(unsigned long long), c->stream));
    launch_argmax(c->n, c->cfg.mode == RAD_MODE_PHYS, c->d_rad, c->d_area, c->d_best, c->stream);
    RAD_CUDA(c, cudaGetLastError());
    unsigned long long best = 0;
    RAD_CUDA(c, cudaMemcpyAsync(&best, c->d_best, sizeof(best), cudaMemcpyDeviceToHost, c->stream));
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    *id = best == ~0ull ? 0u : ~(uint32_t)(best & 0xFFFFFFFFull);
    return RAD_OK;
}

int rad_progress(rad_ctx* c, uint32_t* shots_done, double* initial_power) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    DevState st;
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    RAD_CUDA(c, cudaMemcpy(&st, c->d_state, sizeof(st), cudaMemcpyDeviceToHost));
    if (shots_done) *shots_done = st.shots_done;
    if (initial_power) *initial_power = st.power0;
    return RAD_OK;
}

int rad_set_progress(rad_ctx* c, uint32_t shots_done, double initial_power) {
    if (!c) return RAD_E_INVALID;
    if (!c->n) return fail(c, RAD_E_STATE, "no scene uploaded");
    if (!(initial_power >= 0)) return fail(c, RAD_E_INVALID, "initial power must be >= 0");
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    RAD_CUDA(c, cudaMemcpy(&c->d_state->shots_done, &shots_done, sizeof(shots_done), cudaMemcpyHostToDevice));
    RAD_CUDA(c, cudaMemcpy(&c->d_state->power0, &initial_power, sizeof(initial_power), cudaMemcpyHostToDevice));
    return RAD_OK;
}

int rad_raster_counters(rad_ctx* c, uint64_t* out) {
    if (!c || !out) return RAD_E_INVALID;
    RAD_CUDA(c, cudaStreamSynchronize(c->stream));
    RAD_CUDA(c, cudaMemcpy(out, c->d_state->raster_counters, sizeof(uint64_t) * 8, cudaMemcpyDeviceToHost));
    return RAD_OK;
}

const char* rad_strerror(int status) {
    switch (status) {
        case RAD_OK: return "ok";
        case RAD_E_INVALID: return "invalid argument";
        case RAD_E_CUDA: return "CUDA error";
        case RAD_E_OVERFLOW: return "triangle or bin capacity exceeded";
        case RAD_E_STATE: return "call out of order";
        case RAD_E_NOMEM: return "device allocation failed";
        case RAD_E_TIMEOUT: return "bounded device wait gave up";
        case RAD_E_NOALLOC_LIMIT: return "count * n_patches exceeds RAD_NOALLOC_MAX_SUMS (allocation-free scratch)";
        case RAD_E_NUMERIC: return "non-finite residual";
        default: return "unknown status";
    }
}

const char* rad_last_error(const rad_ctx* c) { return c ? c->err.c_str() : "null context"; }

}  // extern "C"
