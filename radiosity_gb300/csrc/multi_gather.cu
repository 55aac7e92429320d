// Many scenes solved together by learned warm start + BF16 gather under ONE captured CUDA
// graph (rad_multi_gather_*).
//
// Each scene (one rad_ctx, its own stream) is a branch of the graph:
//   1. dense capture: one hemicube per patch (camera, setup, bins, raster + exact reduction,
//      FP32 / BF16 rows) -- the same kernels as rad_dense_capture;
//   2. emission E (3 column-major RHS) from the uploaded unshot energy, and its norms;
//   3. first-shot direct light rho o (M E) by the streaming residual kernel (M = F, or in the
//      shoot form the reciprocity operator (M X)_i = sum_j F_ji A_j X_j / A_i);
//   4. the warm-start features of every patch and the network's forward pass (both on the
//      device), decoded into the guess B0 = E + s * expm1(clip(y, 0, 30));
//   5. the residual of the guess and a check kernel, then a conditional WHILE node whose body
//      is one refinement of rad_gather_solve (BF16 tcgen05 sweeps of the correction, update,
//      FP32 residual with FP64 norms) followed by the check again.  The check kernel sets the
//      node's condition, so every scene iterates on the device until its own relative
//      residual is <= tol (or max_outer refinements): the host launches the graph once.
// The check also stamps the global timer, so each scene's time to tolerance is measured from
// the graph's start.  Without a network the guess is the emission, and a scene's result is
// then bit-identical to rad_gather_solve(E, guess = NULL) with the same tol and sweeps.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <vector>

#include "rad_ctx.cuh"
#include "rad_internal.cuh"

using namespace rad;

namespace {

// Per-scene device scalars and results.
struct SceneDev {
    double enorm2[3];           // ||E_c||^2
    double scale[3];            // s: mean first-shot direct light per channel (+1e-12)
    float lo[3], hi[3];         // bounding box of the patch centres
    double mean_area;
    double residual;            // last relative residual
    double initial_residual;
    uint32_t outer;             // residual evaluations
    uint32_t status;            // 0 running, 1 converged, 2 refinement limit, 3 non-finite residual
    uint32_t err;               // a bounded pipeline wait gave up
    uint32_t pad;
    unsigned long long t_done;  // global timer at the last check
};

struct Fourier {
    float b[8][3];              // feature directions (2 pi p . b_k)
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__global__ void k_mg_stamp(unsigned long long* t0) { *t0 = global_ns(); }

// E (3 x n column-major) from the unshot energy, ||E_c||^2 in FP64, and a cleared SceneDev.
__global__ void __launch_bounds__(256) k_mg_emission(const float4* __restrict__ rad, uint32_t n, float* __restrict__ E,
                                                     SceneDev* sd) {
    __shared__ double red[3][256];
    double a0 = 0, a1 = 0, a2 = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 r = rad[i];
        E[i] = r.x;
        E[(size_t)n + i] = r.y;
        E[(size_t)2 * n + i] = r.z;
        a0 += (double)r.x * r.x;
        a1 += (double)r.y * r.y;
        a2 += (double)r.z * r.z;
    }
    red[0][threadIdx.x] = a0;
    red[1][threadIdx.x] = a1;
    red[2][threadIdx.x] = a2;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int c = 0; c < 3; c++) red[c][threadIdx.x] += red[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int c = 0; c < 3; c++) sd->enorm2[c] = red[c][0];
        sd->outer = 0;
        sd->status = 0;
        sd->residual = 0;
        sd->initial_residual = 0;
        sd->t_done = 0;
    }
}

__device__ __forceinline__ void patch_center_normal_area(const float* __restrict__ verts, uint32_t i, float* c,
                                                         float* nrm, double* area) {
    const float* q = verts + 12 * (size_t)i;
    double v[4][3];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) v[k][d] = q[3 * k + d];
#pragma unroll
    for (int d = 0; d < 3; d++) c[d] = (float)((((v[0][d] + v[1][d]) + v[2][d]) + v[3][d]) / 4.0);
    // normal (v3 - v0) x (v1 - v0), area 0.5 |(v0 - v2) x (v1 - v3)|
    const double a[3] = {v[3][0] - v[0][0], v[3][1] - v[0][1], v[3][2] - v[0][2]};
    const double b[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
    const double nx = a[1] * b[2] - a[2] * b[1], ny = a[2] * b[0] - a[0] * b[2], nz = a[0] * b[1] - a[1] * b[0];
    const double nl = sqrt(nx * nx + ny * ny + nz * nz);
    const double inv = nl > 1e-20 ? 1.0 / nl : 1e20;
    nrm[0] = (float)(nx * inv);
    nrm[1] = (float)(ny * inv);
    nrm[2] = (float)(nz * inv);
    const double d1[3] = {v[0][0] - v[2][0], v[0][1] - v[2][1], v[0][2] - v[2][2]};
    const double d2[3] = {v[1][0] - v[3][0], v[1][1] - v[3][1], v[1][2] - v[3][2]};
    const double cx = d1[1] * d2[2] - d1[2] * d2[1], cy = d1[2] * d2[0] - d1[0] * d2[2],
                 cz = d1[0] * d2[1] - d1[1] * d2[0];
    *area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
}

// The feature normalisations of a scene (one CTA): the centres' bounding box, the mean area
// and the mean first-shot direct light per channel.
__global__ void __launch_bounds__(256) k_mg_stats(const float* __restrict__ verts, const float* __restrict__ direct,
                                                  uint32_t n, SceneDev* sd) {
    __shared__ float slo[3][256], shi[3][256];
    __shared__ double sred[4][256];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double ar = 0, d0 = 0, d1 = 0, d2 = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        float c[3], nrm[3];
        double a;
        patch_center_normal_area(verts, i, c, nrm, &a);
        for (int d = 0; d < 3; d++) {
            lo[d] = fminf(lo[d], c[d]);
            hi[d] = fmaxf(hi[d], c[d]);
        }
        ar += a;
        d0 += direct[i];
        d1 += direct[(size_t)n + i];
        d2 += direct[(size_t)2 * n + i];
    }
    for (int d = 0; d < 3; d++) {
        slo[d][threadIdx.x] = lo[d];
        shi[d][threadIdx.x] = hi[d];
    }
    sred[0][threadIdx.x] = ar;
    sred[1][threadIdx.x] = d0;
    sred[2][threadIdx.x] = d1;
    sred[3][threadIdx.x] = d2;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            for (int d = 0; d < 3; d++) {
                slo[d][threadIdx.x] = fminf(slo[d][threadIdx.x], slo[d][threadIdx.x + o]);
                shi[d][threadIdx.x] = fmaxf(shi[d][threadIdx.x], shi[d][threadIdx.x + o]);
            }
            for (int k = 0; k < 4; k++) sred[k][threadIdx.x] += sred[k][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int d = 0; d < 3; d++) {
            sd->lo[d] = slo[d][0];
            sd->hi[d] = shi[d][0];
            sd->scale[d] = sred[1 + d][0] / (double)n + 1e-12;
        }
        sd->mean_area = sred[0][0] / (double)n;
    }
}

// The 32 warm-start features of every patch (row-major n x 32): normalised centre (3), unit
// normal (3), area / mean area (1), reflectance (3), log1p(direct / s) (3), log1p(E / s) (3),
// sin and cos of 2 pi p . b_k for the 8 feature directions (16).
__global__ void k_mg_features(const float* __restrict__ verts, const float4* __restrict__ rho,
                              const float* __restrict__ E, const float* __restrict__ direct, uint32_t n, Fourier fb,
                              const SceneDev* __restrict__ sd, float* __restrict__ X) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float c[3], nrm[3];
    double a;
    patch_center_normal_area(verts, i, c, nrm, &a);
    float p[3];
    for (int d = 0; d < 3; d++) p[d] = (c[d] - sd->lo[d]) / fmaxf(sd->hi[d] - sd->lo[d], 1e-9f);
    float* x = X + (size_t)i * kMlpIn;
    x[0] = p[0]; x[1] = p[1]; x[2] = p[2];
    x[3] = nrm[0]; x[4] = nrm[1]; x[5] = nrm[2];
    x[6] = (float)(a / sd->mean_area);
    const float4 r = rho[i];
    x[7] = r.x; x[8] = r.y; x[9] = r.z;
    for (int ch = 0; ch < 3; ch++) {
        const float s = (float)sd->scale[ch];
        x[10 + ch] = log1pf(fmaxf(direct[(size_t)ch * n + i], 0.f) / s);
        x[13 + ch] = log1pf(E[(size_t)ch * n + i] / s);
    }
    for (int k = 0; k < 8; k++) {
        const float ph = 6.2831853071795864769f * ((p[0] * fb.b[k][0] + p[1] * fb.b[k][1]) + p[2] * fb.b[k][2]);
        x[16 + k] = sinf(ph);
        x[24 + k] = cosf(ph);
    }
}

// The guess B0 = E + s * expm1(clip(y, 0, 30)), a non-finite output counting as 0.
__global__ void k_mg_decode(const float* __restrict__ E, const float* __restrict__ Y, uint32_t n,
                            const SceneDev* __restrict__ sd, float* __restrict__ B) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int ch = 0; ch < 3; ch++) {
        float y = Y[(size_t)i * kMlpOut + ch];
        y = isfinite(y) ? fminf(fmaxf(y, 0.f), 30.f) : 0.f;
        B[(size_t)ch * n + i] = E[(size_t)ch * n + i] + (float)sd->scale[ch] * expm1f(y);
    }
}

// After a residual: the relative residual max_c ||r_c|| / ||E_c|| (channels with E_c = 0
// skipped, as rad_gather_solve does), the stop decision, and the WHILE node's condition.
__global__ void k_mg_check(const double* __restrict__ nrm, SceneDev* sd, double tol, uint32_t max_outer,
                           cudaGraphConditionalHandle handle) {
    double res = 0;
    bool bad = false;
    for (int c = 0; c < 3; c++) {
        bad = bad || !isfinite(nrm[c]);
        if (sd->enorm2[c] > 0) res = fmax(res, sqrt(nrm[c]) / sqrt(sd->enorm2[c]));
    }
    const uint32_t outer = sd->outer;  // refinements done before this residual
    if (outer == 0) sd->initial_residual = bad ? NAN : res;
    sd->residual = bad ? NAN : res;
    sd->outer = outer + 1;
    uint32_t more = 0;
    if (bad) sd->status = 3;
    else if (res <= tol) sd->status = 1;
    else if (outer >= max_outer) sd->status = 2;
    else more = 1;
    if (!more) sd->t_done = global_ns();
    cudaGraphSetConditional(handle, more);
}

struct Scene {
    rad_ctx* c = nullptr;
    uint32_t n = 0, ld = 0, Rpad = 0, ksplit = 1;
    uint32_t* d_ids = nullptr;
    float *dE = nullptr, *dB = nullptr, *dr = nullptr, *dd = nullptr, *ddir = nullptr;
    float *dpart = nullptr, *dxp = nullptr;
    __nv_bfloat16* d16[2] = {nullptr, nullptr};
    double* dnrm = nullptr;
    float *dX = nullptr, *dact0 = nullptr, *dact1 = nullptr, *dY = nullptr;
    SceneDev* dsd = nullptr;
};

}  // namespace

struct rad_multi_gather {
    std::vector<Scene> scenes;
    const rad_mlp* mlp = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t body_stream = nullptr;
    std::vector<cudaEvent_t> fork, join;
    unsigned long long* d_t0 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    uint32_t sweeps = 4;
    std::string err;
};

namespace {

int mg_fail(rad_multi_gather* m, int code, const char* what) {
    m->err = what;
    return code;
}

// One refinement of rad_gather_solve: correction by `sweeps` BF16 tcgen05 sweeps, update,
// then the FP32 residual and its check.
void enqueue_refinement(const Scene& sc, uint32_t sweeps, double tol, uint32_t max_outer,
                        cudaGraphConditionalHandle handle, cudaStream_t s) {
    rad_ctx* c = sc.c;
    const uint32_t n = sc.n, ld = sc.ld, R = 3;
    const size_t nr = (size_t)n * R;
    if (sweeps == 0) {
        cudaMemcpyAsync(sc.dd, sc.dr, 4 * nr, cudaMemcpyDeviceToDevice, s);
    } else {
        ctx_dense_pack(c, sc.dr, R, sc.d16[0], sc.Rpad, s);
        int cur = 0;
        for (uint32_t k = 0; k < sweeps; k++) {
            TcEpilogue ep{};
            const __nv_bfloat16* M = ctx_dense_sweep(c, ep);
            ep.mode = 1;
            ep.n = n;
            ep.R = R;
            ep.resid = sc.dr;
            ep.out = sc.dd;
            ep.out16 = sc.d16[cur ^ 1];
            ep.ld16 = ld;
            ep.err = &sc.dsd->err;
            ep.partial = sc.dpart;
            ep.ksplit = sc.ksplit;
            launch_gemm_tc(M, n, ld, sc.d16[cur], sc.Rpad, ep, s);
            cur ^= 1;
        }
    }
    launch_axpy(sc.dB, sc.dd, nr, s);
    cudaMemsetAsync(sc.dnrm, 0, 8 * R, s);
    ctx_dense_resid(c, sc.dB, sc.dE, R, sc.dr, sc.dnrm, sc.dxp, &sc.dsd->err, s);
    k_mg_check<<<1, 1, 0, s>>>(sc.dnrm, sc.dsd, tol, max_outer, handle);
}

void free_scene(Scene& sc) {
    cudaFree(sc.d_ids); cudaFree(sc.dE); cudaFree(sc.dB); cudaFree(sc.dr); cudaFree(sc.dd); cudaFree(sc.ddir);
    cudaFree(sc.dpart); cudaFree(sc.dxp); cudaFree(sc.d16[0]); cudaFree(sc.d16[1]); cudaFree(sc.dnrm);
    cudaFree(sc.dX); cudaFree(sc.dact0); cudaFree(sc.dact1); cudaFree(sc.dY); cudaFree(sc.dsd);
    sc = Scene{};
}

}  // namespace

extern "C" {

int rad_multi_gather_destroy(rad_multi_gather* m) {
    if (!m) return RAD_E_INVALID;
    if (m->stream) cudaStreamSynchronize(m->stream);
    if (m->exec) cudaGraphExecDestroy(m->exec);
    if (m->graph) cudaGraphDestroy(m->graph);
    for (auto e : m->fork) cudaEventDestroy(e);
    for (auto e : m->join) cudaEventDestroy(e);
    if (m->e0) cudaEventDestroy(m->e0);
    if (m->e1) cudaEventDestroy(m->e1);
    for (auto& sc : m->scenes) free_scene(sc);
    cudaFree(m->d_t0);
    if (m->body_stream) cudaStreamDestroy(m->body_stream);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return RAD_OK;
}

int rad_multi_gather_create(rad_ctx* const* ctxs, uint32_t count, const rad_mlp* mlp, const double* feature_dirs,
                            double tol, uint32_t max_outer, uint32_t sweeps, uint32_t flags,
                            rad_multi_gather** out) {
    if (!ctxs || count == 0 || !out || !(tol > 0) || sweeps > 64) return RAD_E_INVALID;
    if (flags & ~RAD_DENSE_SHOOT_FORM) return RAD_E_INVALID;
    if (mlp && !feature_dirs) return RAD_E_INVALID;
    *out = nullptr;
    const int dev = ctxs[0]->cfg.device;
    for (uint32_t i = 0; i < count; i++)
        if (!ctxs[i] || !ctxs[i]->n || ctxs[i]->cfg.device != dev || ctxs[i]->cfg.mode != RAD_MODE_PHYS)
            return RAD_E_INVALID;
    if (cudaSetDevice(dev) != cudaSuccess) return RAD_E_CUDA;
    rad_multi_gather* m = new rad_multi_gather();
    m->mlp = mlp;
    m->device = dev;
    m->sweeps = sweeps;
    auto bail = [&](int code) {
        rad_multi_gather_destroy(m);
        return code;
    };
    Fourier fb{};
    if (mlp)
        for (int k = 0; k < 8; k++)
            for (int d = 0; d < 3; d++) fb.b[k][d] = (float)feature_dirs[3 * k + d];
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&m->body_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&m->e0) != cudaSuccess || cudaEventCreate(&m->e1) != cudaSuccess ||
        cudaMalloc(&m->d_t0, sizeof(unsigned long long)) != cudaSuccess)
        return bail(RAD_E_CUDA);
    // per-scene buffers (all allocation happens here, before the capture)
    m->scenes.resize(count);
    for (uint32_t i = 0; i < count; i++) {
        Scene& sc = m->scenes[i];
        rad_ctx* c = ctxs[i];
        sc.c = c;
        int rc = ctx_dense_alloc(c, true, (flags & RAD_DENSE_SHOOT_FORM) != 0);
        if (rc) return bail(rc);
        sc.n = c->n;
        sc.ld = c->dense_ld;
        sc.Rpad = gemm_tc_width(3);
        sc.ksplit = gemm_tc_ksplit(sc.n, sc.ld, sc.Rpad);
        const size_t nr = (size_t)sc.n * 3;
        std::vector<uint32_t> ids(sc.n);
        for (uint32_t k = 0; k < sc.n; k++) ids[k] = k;
        bool ok = cudaMalloc(&sc.d_ids, 4 * (size_t)sc.n) == cudaSuccess &&
                  cudaMemcpy(sc.d_ids, ids.data(), 4 * (size_t)sc.n, cudaMemcpyHostToDevice) == cudaSuccess &&
                  cudaMalloc(&sc.dE, 4 * nr) == cudaSuccess && cudaMalloc(&sc.dB, 4 * nr) == cudaSuccess &&
                  cudaMalloc(&sc.dr, 4 * nr) == cudaSuccess && cudaMalloc(&sc.dd, 4 * nr) == cudaSuccess &&
                  cudaMalloc(&sc.ddir, 4 * nr) == cudaSuccess &&
                  cudaMalloc(&sc.d16[0], 2 * (size_t)sc.Rpad * sc.ld) == cudaSuccess &&
                  cudaMalloc(&sc.d16[1], 2 * (size_t)sc.Rpad * sc.ld) == cudaSuccess &&
                  cudaMemset(sc.d16[0], 0, 2 * (size_t)sc.Rpad * sc.ld) == cudaSuccess &&
                  cudaMemset(sc.d16[1], 0, 2 * (size_t)sc.Rpad * sc.ld) == cudaSuccess &&
                  cudaMalloc(&sc.dnrm, 8 * 3) == cudaSuccess && cudaMalloc(&sc.dsd, sizeof(SceneDev)) == cudaSuccess &&
                  cudaMemset(sc.dsd, 0, sizeof(SceneDev)) == cudaSuccess;
        if (ok && sc.ksplit > 1) ok = cudaMalloc(&sc.dpart, 4 * nr * sc.ksplit) == cudaSuccess;
        if (ok) {
            const size_t xs = sgemm_resid_scratch_floats(3, sc.ld);
            if (xs) ok = cudaMalloc(&sc.dxp, 4 * xs) == cudaSuccess;
        }
        if (ok && mlp)
            ok = cudaMalloc(&sc.dX, 4 * (size_t)sc.n * kMlpIn) == cudaSuccess &&
                 cudaMalloc(&sc.dact0, 4 * (size_t)sc.n * kMlpHidden) == cudaSuccess &&
                 cudaMalloc(&sc.dact1, 4 * (size_t)sc.n * kMlpHidden) == cudaSuccess &&
                 cudaMalloc(&sc.dY, 4 * (size_t)sc.n * kMlpOut) == cudaSuccess;
        if (!ok) return bail(mg_fail(m, RAD_E_NOMEM, "multi-gather buffers"));
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(RAD_E_CUDA);
    }
    m->fork.resize(count);
    m->join.resize(count);
    for (uint32_t i = 0; i < count; i++)
        if (cudaEventCreateWithFlags(&m->fork[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&m->join[i], cudaEventDisableTiming) != cudaSuccess)
            return bail(RAD_E_CUDA);
    // capture: the stamp, then one branch per scene on its context's stream
    if (cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return bail(RAD_E_CUDA);
    k_mg_stamp<<<1, 1, 0, m->stream>>>(m->d_t0);
    bool ok = true;
    for (uint32_t i = 0; i < count && ok; i++) {
        Scene& sc = m->scenes[i];
        rad_ctx* c = sc.c;
        cudaStream_t s = c->stream;
        const uint32_t n = sc.n, ld = sc.ld;
        cudaEventRecord(m->fork[i], m->stream);
        cudaStreamWaitEvent(s, m->fork[i], 0);
        ctx_enqueue_dense_capture(c, sc.d_ids, s);
        k_mg_emission<<<1, 256, 0, s>>>(c->d_rad, n, sc.dE, sc.dsd);
        if (mlp) {
            cudaMemsetAsync(sc.dnrm, 0, 8 * 3, s);
            ctx_dense_resid(c, sc.dE, sc.dE, 3, sc.ddir, sc.dnrm, sc.dxp, &sc.dsd->err, s);
            k_mg_stats<<<1, 256, 0, s>>>(c->d_verts, sc.ddir, n, sc.dsd);
            k_mg_features<<<(n + 127) / 128, 128, 0, s>>>(c->d_verts, c->d_rho, sc.dE, sc.ddir, n, fb, sc.dsd, sc.dX);
            mlp_forward_device(mlp, sc.dX, n, sc.dact0, sc.dact1, sc.dY, s);
            k_mg_decode<<<(n + 127) / 128, 128, 0, s>>>(sc.dE, sc.dY, n, sc.dsd, sc.dB);
        } else {
            cudaMemcpyAsync(sc.dB, sc.dE, 4 * (size_t)n * 3, cudaMemcpyDeviceToDevice, s);
        }
        // the guess's residual and check, then the refinement loop as a conditional WHILE node
        cudaGraph_t g = nullptr;
        cudaStreamCaptureStatus cs;
        cudaGraphConditionalHandle handle;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        ok = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps) == cudaSuccess &&
             cs == cudaStreamCaptureStatusActive &&
             cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
        if (!ok) break;
        cudaMemsetAsync(sc.dnrm, 0, 8 * 3, s);
        ctx_dense_resid(c, sc.dB, sc.dE, 3, sc.dr, sc.dnrm, sc.dxp, &sc.dsd->err, s);
        k_mg_check<<<1, 1, 0, s>>>(sc.dnrm, sc.dsd, tol, max_outer, handle);
        ok = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps) == cudaSuccess;
        if (!ok) break;
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        ok = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp) == cudaSuccess &&
             cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
        if (!ok) break;
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(m->body_stream, body, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (!ok) break;
        enqueue_refinement(sc, sweeps, tol, max_outer, handle, m->body_stream);
        ok = cudaStreamEndCapture(m->body_stream, &body) == cudaSuccess;
        cudaEventRecord(m->join[i], s);
        cudaStreamWaitEvent(m->stream, m->join[i], 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(m->stream, &graph);
    m->graph = graph;
    if (!ok || ec != cudaSuccess) {
        cudaGetLastError();
        return bail(RAD_E_CUDA);
    }
    if (cudaGraphInstantiate(&m->exec, m->graph, 0) != cudaSuccess) return bail(RAD_E_CUDA);
    *out = m;
    return RAD_OK;
}

int rad_multi_gather_run(rad_multi_gather* m, double* device_ms, double* scene_ms, uint32_t* outer,
                         double* residual, double* initial_residual, uint32_t* status) {
    if (!m) return RAD_E_INVALID;
    if (cudaSetDevice(m->device) != cudaSuccess) return RAD_E_CUDA;
    if (cudaEventRecord(m->e0, m->stream) != cudaSuccess || cudaGraphLaunch(m->exec, m->stream) != cudaSuccess ||
        cudaEventRecord(m->e1, m->stream) != cudaSuccess || cudaStreamSynchronize(m->stream) != cudaSuccess)
        return RAD_E_CUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, m->e0, m->e1);
    if (device_ms) *device_ms = ms;
    unsigned long long t0 = 0;
    if (cudaMemcpy(&t0, m->d_t0, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return RAD_E_CUDA;
    int rc = RAD_OK;
    for (size_t i = 0; i < m->scenes.size(); i++) {
        SceneDev sd;
        DevState st;
        if (cudaMemcpy(&sd, m->scenes[i].dsd, sizeof(sd), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&st, m->scenes[i].c->d_aux, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess)
            return RAD_E_CUDA;
        if (scene_ms) scene_ms[i] = sd.t_done > t0 ? (double)(sd.t_done - t0) * 1e-6 : 0.0;
        if (outer) outer[i] = sd.outer;
        if (residual) residual[i] = sd.residual;
        if (initial_residual) initial_residual[i] = sd.initial_residual;
        if (status) status[i] = sd.status;
        if (st.overflow) rc = RAD_E_OVERFLOW;
        else if (sd.err && rc == RAD_OK) rc = RAD_E_TIMEOUT;
        else if (sd.status == 3 && rc == RAD_OK) rc = RAD_E_NUMERIC;
    }
    for (auto& sc : m->scenes) sc.c->dense_ready = true;
    return rc;
}

int rad_multi_gather_result(rad_multi_gather* m, uint32_t index, float* radiosity) {
    if (!m || !radiosity || index >= m->scenes.size()) return RAD_E_INVALID;
    const Scene& sc = m->scenes[index];
    return cudaMemcpy(radiosity, sc.dB, 4 * (size_t)sc.n * 3, cudaMemcpyDeviceToHost) == cudaSuccess ? RAD_OK
                                                                                                      : RAD_E_CUDA;
}

}  // extern "C"
