// Allocation-free form-factor rows: rad_reduce_items_noalloc.
//
// Some callers cannot allocate device memory: a host application whose device
// memory is owned by another allocator's pool (a framework's caching allocator
// that has reserved most of the GPU, so a raw cudaMalloc fails or fragments it),
// or a frame loop with a fixed memory budget that must not allocate per call.
// They own their input and output buffers and only need the computation.  This
// entry point is a variant of the item-buffer reduction (k_reduce_items in
// raster.cu) that keeps its only scratch, the exact 64-bit per-patch sums, in
// the file-scope device array below; it computes the delta form factors on the
// fly instead of reading the context's table, so it needs no context either.
//
// Scratch: kNoAllocMaxSums uint64 sums = 8 MiB, held by every GPU that loads the
// library until the process exits.  A call may process count * n_patches <=
// kNoAllocMaxSums sums; larger requests return RAD_E_NOALLOC_LIMIT.
// Every call shares the array: each call clears the count * n_patches sums it
// uses before accumulating, so a call never sees a previous call's contents;
// calls that overlap on the GPU (different streams or host threads) race on it.
// The device address of the array is looked up with cudaGetSymbolAddress once per
// device, with that device current, on the first call made on that device.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "radiosity.h"

namespace {

constexpr size_t kNoAllocMaxSums = RAD_NOALLOC_MAX_SUMS;
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) unsigned long long g_noalloc_sums[kNoAllocMaxSums];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_sums on the current device (looked up once per device).
cudaError_t noalloc_scratch(unsigned long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_sums);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned long long*>(g_noalloc_ptr[dev]);
    return cudaSuccess;
}

// Delta form factor of texel i of the 2W x 1.5W layout (source/FormFactors.cpp:23-67,
// :295-314), same float operations as the table the context builds.
__device__ float noalloc_ff(uint32_t W, uint32_t i) {
    const uint32_t H = W, TW = 2 * W;
    const int n = (int)W;
    const float PI = 3.1415926535897932384626433832795028841931f;
    float hpw = (1.0f / n);
    float pix = (2.0f / n);
    pix *= pix;
    uint32_t x = i % TW, y = i / TW, k;
    bool front = false;
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
    if (front) {
        float dx = ((tx - n / 2) / (n / 2.0f)) + hpw;
        float dy = ((ty - n / 2) / (n / 2.0f)) + hpw;
        float f = (dx * dx + dy * dy + 1);
        f *= f * PI;
        return pix / f;
    }
    float dx = (tx - n / 2) / (n / 2.0f) + hpw;
    float dy = (n / 2 - 1 - ty) / (n / 2.0f) + hpw;
    float f = (dx * dx + dy * dy + 1);
    f *= f * PI;
    return (pix * (dy + hpw)) / f;
}

__global__ void k_noalloc_clear(unsigned long long* sums, size_t total) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        sums[i] = 0;
}

// Grid-stride over the count * 3W^2 texels; the stride is a whole number of blocks, so the
// lanes of a warp run the same iterations and the warp-wide match below sees all 32 lanes.
__global__ void k_noalloc_reduce(const uint32_t* __restrict__ items, uint32_t count, uint32_t W, uint32_t n,
                                 unsigned long long* sums) {
    const uint32_t res = 3 * W * W;
    const size_t total = (size_t)count * res;
    const int lane = threadIdx.x & 31;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < total; base += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = base + threadIdx.x;
        const uint32_t it = idx < total ? items[idx] : 0u;
        const bool has = it != 0 && it <= n;
        const uint32_t hi = (uint32_t)(idx / res), pix = (uint32_t)(idx % res);
        unsigned long long q = 0;
        if (has) q = __float2ull_rz(noalloc_ff(W, pix) * 0x1p61f);
        // one warp may span several images (12 texels each at W = 2): the key holds the image
        // index and the patch id
        const unsigned long long key = has ? ((unsigned long long)hi << 32) | (it - 1) : ~0ull;
        const unsigned m = __match_any_sync(0xffffffffu, key);
        const uint32_t a = (uint32_t)(q & 0x1FFFFFull), b = (uint32_t)((q >> 21) & 0x1FFFFFull),
                       c = (uint32_t)(q >> 42);
        const uint32_t sa = __reduce_add_sync(m, a), sb = __reduce_add_sync(m, b), sc = __reduce_add_sync(m, c);
        const unsigned long long sum =
            (unsigned long long)sa + ((unsigned long long)sb << 21) + ((unsigned long long)sc << 42);
        if (has && lane == __ffs(m) - 1) atomicAdd(&sums[(size_t)hi * n + (it - 1)], sum);
    }
}

__global__ void k_noalloc_to_float(const unsigned long long* __restrict__ sums, size_t total, float* out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __ull2float_rn(sums[i]) * 0x1p-61f;
}

}  // namespace

extern "C" int rad_reduce_items_noalloc(const uint32_t* d_items, uint32_t count, uint32_t hemicube_side,
                                        uint32_t n_patches, float* d_ff_rows, void* stream) {
    if (!d_items || !d_ff_rows || count == 0 || n_patches == 0) return RAD_E_INVALID;
    if (hemicube_side < 2 || hemicube_side > 2048 || (hemicube_side & 1u)) return RAD_E_INVALID;
    const size_t sums = (size_t)count * n_patches;
    if (sums > kNoAllocMaxSums) return RAD_E_NOALLOC_LIMIT;
    unsigned long long* scratch = nullptr;
    if (noalloc_scratch(&scratch) != cudaSuccess) return RAD_E_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t pixels = (size_t)count * 3 * hemicube_side * hemicube_side;
    k_noalloc_clear<<<152 * 4, 256, 0, s>>>(scratch, sums);
    const size_t blocks = (pixels + 255) / 256;
    const unsigned grid = blocks < (size_t)152 * 64 ? (unsigned)blocks : 152u * 64u;  // grid-stride beyond
    k_noalloc_reduce<<<grid, 256, 0, s>>>(d_items, count, hemicube_side, n_patches, scratch);
    k_noalloc_to_float<<<152 * 4, 256, 0, s>>>(scratch, sums, d_ff_rows);
    if (cudaGetLastError() != cudaSuccess) return RAD_E_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RAD_E_CUDA;
    return RAD_OK;
}
