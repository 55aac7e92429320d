// The solver context (struct rad_ctx of include/radiosity.h) and the context helpers that
// the C ABI's translation units share.  Private to the library.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

#include "radiosity.h"
#include "rad_internal.cuh"

struct BatchBuf {
    rad::Batch b{};
    uint32_t cap_k = 0;
    bool has_items = false;
};

struct rad_ctx {
    rad_config cfg{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    rad::Geo geo{};
    uint32_t n = 0;
    float* d_verts = nullptr;
    float4* d_color = nullptr;
    float4* d_rho = nullptr;
    float4* d_rad = nullptr;
    float4* d_illum = nullptr;
    float* d_area = nullptr;
    float* d_gbox = nullptr;       // bounding box of each group of 128 patches (k_setup's CTAs), 6 floats
    uint32_t* d_nb = nullptr;      // display neighbours, N x 8 (rad_upload_neighbours)
    float* d_shade = nullptr;      // display colour scratch, 2 x N x 12 (rad_display_colors)
    unsigned long long* d_best = nullptr;  // argmax key (rad_highest_patch)
    float* d_fftab = nullptr;
    rad::BinInfo* d_bins = nullptr;
    rad::DevState* d_state = nullptr;   // shoot loop state
    rad::DevState* d_aux = nullptr;     // state for the one-off entry points
    uint32_t* h_flag = nullptr;    // pinned stop flag
    float* d_f3 = nullptr;         // device scratch for the host's float3 arrays, 2 x 3N floats
    BatchBuf shoot;                // K = hemicubes_count
    BatchBuf aux;                  // one-off calls, grown on demand
    float* d_rows = nullptr;       // float rows for ff_rows / reduce
    size_t rows_cap = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    // dense form factors (rad_dense_capture)
    float* d_F32 = nullptr;
    __nv_bfloat16* d_F16 = nullptr;
    float* d_scale = nullptr;
    uint32_t dense_ld = 0;
    bool dense_ready = false;
    // shoot form (RAD_DENSE_SHOOT_FORM): transposed rows and area weights
    bool dense_shoot = false;
    float* d_F32T = nullptr;
    __nv_bfloat16* d_F16T = nullptr;
    float* d_inv_area = nullptr;   // 1 / A
    float* d_wT = nullptr;         // scale o A
};


// rad_api.cu
int ctx_fail(rad_ctx* ctx, int code, const char* msg);
// Batch buffers for K hemicubes (grown on demand; K <= the buffers' capacity reuses them).
int ctx_alloc_batch(rad_ctx* c, BatchBuf& bb, uint32_t K, bool items);
// Dense form-factor storage (BF16 rows + scales, and FP32 rows when fp32; with shoot, the
// transposed copies and area weights of the shoot form) and the aux batch of the capture; no
// capture yet.
int ctx_dense_alloc(rad_ctx* c, bool fp32, bool shoot = false);
// The dense capture's kernels on `s` for rows [0, n) with shooter ids d_ids (0..n-1): no
// allocation, no synchronisation (graph-capturable).  ctx_dense_alloc first.
void ctx_enqueue_dense_capture(rad_ctx* c, const uint32_t* d_ids, cudaStream_t s);
uint32_t ctx_dense_chunk(const rad_ctx* c);

// The captured system's operator M in the form chosen at allocation:
//   gather form  (M X)_i = sum_j F_ij X_j                 B = E + rho o (F B)
//   shoot form   (M X)_i = (sum_j F_ji A_j X_j) / A_i     the progressive shooter's fixed point
// r = E + rho o (M X) - X on the FP32 rows (norms into nrm when given).
void ctx_dense_resid(const rad_ctx* c, const float* X, const float* E, uint32_t R, float* r, double* nrm,
                     float* scratch, uint32_t* err, cudaStream_t s);
// The BF16 right-hand sides of a sweep from X (column-major n x R).
void ctx_dense_pack(const rad_ctx* c, const float* X, uint32_t R, __nv_bfloat16* Xt, uint32_t Rpad,
                    cudaStream_t s);
// Sets the sweep epilogue's scale / wscale / rho for the form; returns the BF16 matrix.
const __nv_bfloat16* ctx_dense_sweep(const rad_ctx* c, rad::TcEpilogue& ep);
