// Internal types shared by the solver's translation units.
//
// Device data layout (one rad_ctx, all resident in HBM):
//   scene      verts   float[N*12]  4 corners per patch, as ModelContainer::getVertices
//              color   float4[N]    rgb of Patch::getColor
//              rho     float4[N]    per-channel reflectance (PHYS)
//              area    float[N]     quad area (PHYS)
//              rad     float4[N]    Patch::radiosity   (unshot energy)
//              illum   float4[N]    Patch::illumination (shot energy)
//   hemicube   fftab   float[3W^2]  delta form factors, texture layout, ONE copy
//   batch (K)  shooters/valid/saved/mvp/frame, triangle records, per-bin lists,
//              Fq uint64[K*N] exact form-factor sums, optional item buffers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rad {

constexpr float kGuard = 1024.0f;       // guard-band clip |x|,|y| <= 1024 w
constexpr float kReflectivity = 0.3f;   // REFLECTIVITY, source/Patch.h:13
constexpr uint32_t kDeadTri = 0xFFFFFFFFu;
constexpr int kMaxK = 1024;

// One rasterisable record: up to two triangles of one patch that share vertex 0,
// A = (v0, v1, v2) and B = (v0, v2, v3).  An unclipped patch quad is one record (its
// two triangles, source/ModelContainer.cpp:112-117); a clipped triangle's fan is
// packed two triangles per record.  Hemicube-local 24.8 fixed-point window coordinates.
// Each triangle keeps its own depth plane; the plane's constant term is rebuilt from
// d0 exactly as it was computed: c0 = (d0 + gx*ox) + gy*oy with gx = ax / 256.
struct __align__(16) TriRec {
    int32_t X[4], Y[4];     // v3 = v2 when B is absent
    float d0;               // 1/w at v0
    float ax[2], ay[2];     // plane gradients x256 of A and B: D = (c0 + ax*(px-sx)) + ay*(py-sy)
    uint32_t id;            // patch index, kDeadTri for an unused slot
    uint32_t bx, by;        // union pixel bbox clamped to the face scissor:
                            // bx = px0 | px1 << 12 | face << 24 | A << 28 | B << 29, by = py0 | py1 << 12
};
static_assert(sizeof(TriRec) == 64, "TriRec layout");
constexpr uint32_t kRecA = 1u << 28, kRecB = 1u << 29;
__host__ __device__ inline int rec_px0(const TriRec& t) { return (int)(t.bx & 0xFFFu); }
__host__ __device__ inline int rec_px1(const TriRec& t) { return (int)((t.bx >> 12) & 0xFFFu); }
__host__ __device__ inline int rec_face(const TriRec& t) { return (int)((t.bx >> 24) & 7u); }
__host__ __device__ inline int rec_py0(const TriRec& t) { return (int)(t.by & 0xFFFu); }
__host__ __device__ inline int rec_py1(const TriRec& t) { return (int)((t.by >> 12) & 0xFFFu); }

struct BinInfo {
    int16_t x0, y0, w, h;   // hemicube-local pixel rectangle
    int32_t face;
};

struct FaceInfo {
    int vp[4];              // viewport x,y,w,h (hemicube-local)
    int sc[4];              // scissor x,y,w,h (hemicube-local)
    int bin_base, bins_x, bins_y, pad;
};

// Per-context constants passed by value to kernels.
struct Geo {
    uint32_t W, TW, TH, RES;   // W, 2W, 1.5W, 3W^2
    uint32_t n;                // patches
    uint32_t nb;               // bins per hemicube
    uint32_t tile;             // bin side
    uint32_t mode;             // rad_mode
    uint32_t small_max;        // span-raster threshold (box clamped to a bin, pixels)
    uint32_t tile_shift;       // log2(tile)
    FaceInfo face[5];
    float proj[16];            // Perspective(90,1,0.01,1000), column-major
};

// Device-side loop state (one per context).
struct DevState {
    uint32_t stopped;
    uint32_t shots_done;
    uint32_t overflow;
    uint32_t reserved;
    float last_energy[4];
    double residual;
    double power0;
    double hemicubes;
    uint32_t timeouts;
    uint32_t pad[3];
    // raster counters (filled when counting is on): record-bin pairs, small records, small box px,
    // big records, big stamps in bbox, stamps visited, stamps fully inside, big pixels plotted;
    // then (phase profiling only) SM cycles summed over warps per raster phase: bin set-up,
    // record staging, row ownership, row spans, pixel stream, pass barrier, big records and
    // chunk barrier, bin end
    unsigned long long raster_counters[16];
};

// Device pointers of one batch of K hemicubes.
struct Batch {
    uint32_t K;
    uint32_t tri_cap;            // K * tri_cap_h
    uint32_t list_cap;
    uint32_t tri_cap_h;          // triangle records per hemicube
    uint32_t list_cap_h;         // bin references per hemicube: hemicube h's lists are in
                                 // [h * list_cap_h, (h + 1) * list_cap_h) of bin_list
    uint32_t* tri_counts;        // K per-hemicube record counts
    uint32_t* shooters;          // K
    uint32_t* valid;             // K
    float4* saved;               // K
    float* mvp;                  // K*5*16
    float* frame;                // K*8 (center xyz, normal xyz)
    TriRec* tris;                // tri_cap records: hemicube h owns [h*tri_cap_h, (h+1)*tri_cap_h)
    uint32_t* bin_count;         // K*nb
    uint32_t* bin_offset;        // K*nb
    uint32_t* bin_fill;          // K*nb
    uint32_t* bin_list;          // list_cap
    unsigned long long* Fq;      // K*N exact sums (scale 2^61)
    uint32_t* items;             // K*RES or null
    const BinInfo* bins;         // nb
    // PHYS selection scratch
    uint32_t* sel_hist;          // 2048 (cleared by the pick kernel after use)
    uint32_t* sel_ctrl;          // 8
    uint32_t* sel_keys;          // N
    unsigned long long* sel_sure;  // K
    unsigned long long* sel_bnd;   // N
    double* partials;            // kUpdateBlocks FP64 residual partials
};
constexpr int kUpdateBlocks = 152 * 8;

// Launchers (raster.cu / shoot.cu).  All run on `s`.
void launch_camera(const Geo& g, const Batch& b, const float* verts, const float4* rad, DevState* st,
                   cudaStream_t s);
// gbox: bounding box (min xyz, max xyz) of each group of 128 patches (launch_group_boxes)
void launch_setup(const Geo& g, const Batch& b, const float* verts, const float* gbox, DevState* st, cudaStream_t s);
void launch_group_boxes(const float* verts, uint32_t n, float* gbox, cudaStream_t s);
void launch_bins(const Geo& g, const Batch& b, DevState* st, cudaStream_t s);
cudaError_t raster_init();  // per device, before the first launch_raster (dynamic shared memory limits)
void launch_raster(const Geo& g, const Batch& b, const float* fftab, DevState* st, bool write_items,
                   bool fused_reduce, cudaStream_t s, bool count = false, bool phases = false);
void launch_reduce_items(const Geo& g, const Batch& b, const float* fftab, uint32_t count, cudaStream_t s);
void launch_fq_to_float(const Geo& g, const Batch& b, uint32_t count, float* out, cudaStream_t s);
void launch_select(const Geo& g, const Batch& b, const float4* rad, const float* area, DevState* st,
                   cudaStream_t s);
void launch_update(const Geo& g, const Batch& b, const float4* color, const float4* rho, const float* area,
                   float4* rad, DevState* st, cudaStream_t s);
void launch_emitters(const Geo& g, const Batch& b, float4* rad, float4* illum, const float* area,
                     double tol, double* partials, DevState* st, cudaStream_t s);
void launch_areas(const float* verts, uint32_t n, float* area, cudaStream_t s);
void launch_f3_to_f4(const float* src, float4* dst, uint32_t n, cudaStream_t s);
void launch_f4_to_f3(const float4* src, float* dst, uint32_t n, cudaStream_t s);
// display.cu
void launch_shade(uint32_t n, const uint32_t* nb, const float4* color, const float4* rad, const float4* illum,
                  float* colors, float* radiative, cudaStream_t s);
void launch_argmax(uint32_t n, bool phys, const float4* rad, const float* area, unsigned long long* best,
                   cudaStream_t s);

// dense.cu
}  // namespace rad
#include <cuda_bf16.h>
namespace rad {
// Epilogue of k_gemm_tc for C = A Bt^T (row = A row, c = Bt row):
//   mode 0: out[c][row] = scale[row] * acc                       (column-major, + BF16 copy)
//   mode 1: out[c][row] = resid[c][row] + rho[row].c * (scale * acc); its BF16 copy holds
//           out * wscale[row] (wscale may be null: 1)
//   mode 2: y = max(acc + bias[c], 0): BF16 out16r[row][c] (row-major, ldr) and out16[c][row]
//   mode 3: out[row][c] = acc + bias[c]                          (row-major FP32, stride R)
//   mode 4: y = acc if mask[row][c] > 0 else 0 (mask BF16 row-major, ldm): BF16 as mode 2
//   mode 5: out[row][c] = acc                                    (row-major FP32, stride ldr)
// Modes 2-5 are the warm-start network's layers (forward, input gradient, weight gradient).
struct TcEpilogue {
    int mode;
    uint32_t n, R;             // rows, output columns
    const float* scale;        // n (may be null: 1)
    const float4* rho;         // n (mode 1)
    const float* resid;        // R x n column-major (mode 1)
    float* out;                // modes 0, 1: R x n column-major; modes 3, 5: row-major
    __nv_bfloat16* out16;      // R x ld16 (next operand), may be null
    uint32_t ld16;
    uint32_t* err;
    float* partial;            // split-K partial sums, ksplit x R x n (null: one split, fused epilogue)
    uint32_t ksplit;           // K splits (gemm_tc_ksplit); > 1 only with `partial`
    const float* bias;         // R (modes 2, 3)
    __nv_bfloat16* out16r;     // row-major BF16 output (modes 2, 4), row stride ldr
    uint32_t ldr;
    const __nv_bfloat16* mask; // mode 4, row stride ldm
    uint32_t ldm;
    const float* wscale;       // n (mode 1, may be null)
};
void launch_dense_rows(unsigned long long* Fq, uint32_t count, uint32_t n, uint32_t ld, uint32_t first,
                       float* F32, __nv_bfloat16* F16, float* scale, cudaStream_t s);
// r = E + rho o (inv_a o (F (w o X))) - X (w, inv_a may be null: ones), `scratch` holding
// sgemm_resid_scratch_floats(R, ld) floats.  R <= 4 takes the streaming kernel (scratch: the
// padded right-hand sides), which sets *err (when given) if one of its bounded pipeline waits
// timed out; larger R the tiled kernel (scratch: its split-K partial sums; when it is 0 or
// null the tiled kernel runs unsplit).
size_t sgemm_resid_scratch_floats(uint32_t R, uint32_t ld);
// resid.cu: the streaming kernel of the R <= kResidStreamRhs residual (scratch: kResidStreamRhs
// x ld floats) and its shared-memory limits (before the first launch).
constexpr uint32_t kResidStreamRhs = 4;
void launch_resid_stream(const float* F, uint32_t n, uint32_t ld, const float* X, const float* E, const float4* rho,
                         uint32_t R, float* r, double* nrm, float* scratch, uint32_t* err, cudaStream_t s,
                         const float* w, const float* inv_a);
cudaError_t resid_stream_init();
// One bounded mbarrier wait that nothing completes: sets *err after limit_ns.
int launch_wait_selftest(uint32_t* err, unsigned long long limit_ns, cudaStream_t s);
void launch_sgemm_resid(const float* F, uint32_t n, uint32_t ld, const float* X, const float* E, const float4* rho,
                        uint32_t R, float* r, double* nrm, float* scratch, uint32_t* err, cudaStream_t s,
                        const float* w = nullptr, const float* inv_a = nullptr);
void launch_shoot_resid(const float* F, uint32_t n, uint32_t ld, const float* X, const float* E, const float4* rho,
                        const float* area, uint32_t R, double* acc, float* r, cudaStream_t s);
void launch_pack_bf16(const float* X, uint32_t n, uint32_t R, uint32_t ld, __nv_bfloat16* Xt, uint32_t Rpad,
                      cudaStream_t s, const float* w = nullptr);
// Shoot-form operands from the captured rows: F32T / F16T = transposes (F32 may be null),
// inv_a = 1 / A, w = scale o A.
void launch_shoot_form(uint32_t n, uint32_t ld, const float* F32, float* F32T, const __nv_bfloat16* F16,
                       __nv_bfloat16* F16T, const float* area, const float* scale, float* inv_a, float* w,
                       cudaStream_t s);
void launch_axpy(float* y, const float* x, size_t total, cudaStream_t s);
int launch_gemm_tc(const __nv_bfloat16* A, uint32_t n, uint32_t ld, const __nv_bfloat16* Bt, uint32_t Rpad,
                   const TcEpilogue& ep, cudaStream_t s);
uint32_t gemm_tc_width(uint32_t R);
cudaError_t dense_init();  // per device, before the first residual / tcgen05 launch
uint32_t gemm_tc_ksplit(uint32_t n, uint32_t ld, uint32_t R);  // K splits that fill the GPU best
void launch_fftab(uint32_t W, float* fftab, cudaStream_t s);

}  // namespace rad

// mlp.cu: the warm-start network's forward pass on device rows (no allocation, no
// synchronisation): X (P x 32, row-major) -> Y (P x 3); act0 / act1 hold P x 128 floats each.
struct rad_mlp;
namespace rad {
void mlp_forward_device(const rad_mlp* m, const float* X, uint32_t P, float* act0, float* act1, float* Y,
                        cudaStream_t s);
constexpr int kMlpIn = 32, kMlpHidden = 128, kMlpOut = 3;
}  // namespace rad
