// Display colours and single-patch selection on the device-resident state.
//
//   k_shade   Colors::smoothShadePatch (source/Colors.cpp:198-262) for every patch:
//             the colour of each of the 4 corners is the mean of the patch's and three
//             neighbours' colour x (illumination + radiosity), as the reference fills
//             its colour VBO after each batch of shots (source/Main.cpp:1318-1340); and
//             the "radiative" VBO, the patch's radiosity repeated at its 4 corners
//             (source/Main.cpp:1346-1372).  Outputs go to device buffers, N x 12 floats
//             (the VBO layout: corner 1..4 x rgb), in place of the mapped GL buffers.
//   k_argmax  ModelContainer::getHighestRadiosityPatchId (source/ModelContainer.cpp:222-237):
//             the first patch with the largest |radiosity|^2 (PHYS: largest unshot power).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "rad_internal.cuh"

namespace rad {

// c * (illumination + radiosity), Vector3f component-wise operators (source/Vector.h:428-431).
__device__ __forceinline__ float3 shade_term(const float4* __restrict__ color, const float4* __restrict__ rad,
                                             const float4* __restrict__ illum, uint32_t j) {
    const float4 c = color[j], r = rad[j], l = illum[j];
    return make_float3(c.x * (l.x + r.x), c.y * (l.y + r.y), c.z * (l.z + r.z));
}

// ((s + a) + b) + c, then Vector3::operator/(4): multiplication by 1/4 (source/Vector.h:448-452).
__device__ __forceinline__ float3 corner(float3 s, float3 a, float3 b, float3 c) {
    float3 o = s;
    o.x += a.x; o.y += a.y; o.z += a.z;
    o.x += b.x; o.y += b.y; o.z += b.z;
    o.x += c.x; o.y += c.y; o.z += c.z;
    const float t = 1.0f / 4.0f;
    return make_float3(o.x * t, o.y * t, o.z * t);
}

__global__ void k_shade(uint32_t n, const uint32_t* __restrict__ nb, const float4* __restrict__ color,
                        const float4* __restrict__ rad, const float4* __restrict__ illum, float* __restrict__ colors,
                        float* __restrict__ radiative) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (colors) {
            const uint4 n03 = reinterpret_cast<const uint4*>(nb)[2 * (size_t)i];
            const uint4 n47 = reinterpret_cast<const uint4*>(nb)[2 * (size_t)i + 1];
            const float3 s = shade_term(color, rad, illum, i);
            const float3 s0 = shade_term(color, rad, illum, n03.x), s1 = shade_term(color, rad, illum, n03.y);
            const float3 s2 = shade_term(color, rad, illum, n03.z), s3 = shade_term(color, rad, illum, n03.w);
            const float3 s4 = shade_term(color, rad, illum, n47.x), s5 = shade_term(color, rad, illum, n47.y);
            const float3 s6 = shade_term(color, rad, illum, n47.z), s7 = shade_term(color, rad, illum, n47.w);
            const float3 lt = corner(s, s7, s0, s1);  // upper left: left, upper left, upper
            const float3 rt = corner(s, s1, s2, s3);  // upper right
            const float3 rb = corner(s, s3, s4, s5);  // lower right
            const float3 lb = corner(s, s5, s6, s7);  // lower left
            float* o = colors + 12 * (size_t)i;   // VBO order: lb, rb, rt, lt (source/Colors.cpp:257-260)
            o[0] = lb.x; o[1] = lb.y; o[2] = lb.z;
            o[3] = rb.x; o[4] = rb.y; o[5] = rb.z;
            o[6] = rt.x; o[7] = rt.y; o[8] = rt.z;
            o[9] = lt.x; o[10] = lt.y; o[11] = lt.z;
        }
        if (radiative) {
            const float4 r = rad[i];
            float* o = radiative + 12 * (size_t)i;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                o[3 * k] = r.x;
                o[3 * k + 1] = r.y;
                o[3 * k + 2] = r.z;
            }
        }
    }
}

void launch_shade(uint32_t n, const uint32_t* nb, const float4* color, const float4* rad, const float4* illum,
                  float* colors, float* radiative, cudaStream_t s) {
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 152u * 8u);
    k_shade<<<blocks, 256, 0, s>>>(n, nb, color, rad, illum, colors, radiative);
}

// Order-preserving map of a float to uint32 (larger float -> larger integer).
__device__ __forceinline__ uint32_t ordered_bits(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// One packed key per patch, (ordered value << 32) | ~index, reduced with a 64-bit
// atomicMax: the largest value wins and among equal values the smallest index.  The
// reference scans patches in order with `max == NULL || v > max_v` (a strict test, first
// patch taken unconditionally): later equal values do not replace, and a NaN never
// replaces nor is replaced once it is the current maximum.  So patch 0 is the answer when
// its value is NaN, and other NaN patches never are.
__global__ void k_argmax(uint32_t n, uint32_t phys, const float4* __restrict__ rad, const float* __restrict__ area,
                         unsigned long long* best) {
    unsigned long long mine = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r = rad[i];
        // + 0.0f turns -0 into +0: the reference's > treats the two zeros as equal
        const float v = (phys ? ((r.x + r.y) + r.z) * area[i] : (r.x * r.x + r.y * r.y) + r.z * r.z) + 0.0f;
        unsigned long long k;
        if (v != v) k = i == 0 ? ~0ull : 0ull;  // NaN: patch 0 wins outright, others never
        else k = ((unsigned long long)ordered_bits(v) << 32) | (uint32_t)~i;
        mine = k > mine ? k : mine;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, mine, o);
        mine = other > mine ? other : mine;
    }
    if ((threadIdx.x & 31) == 0 && mine) atomicMax(best, mine);
}

void launch_argmax(uint32_t n, bool phys, const float4* rad, const float* area, unsigned long long* best,
                   cudaStream_t s) {
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 152u * 4u);
    k_argmax<<<blocks, 256, 0, s>>>(n, phys ? 1u : 0u, rad, area, best);
}

}  // namespace rad
