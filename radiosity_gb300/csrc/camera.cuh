// Hemicube face cameras on the device.
//
// Follows, operation for operation, Patch::getCenter/getNormal/getUp
// (source/Patch.cpp:253-276), Camera::lookFromPatch (source/Camera.cpp:19-52),
// CGLTransform::LookAt (source/Transform.cpp:127-156) and the Matrix4f products
// (source/Vector.cpp:445-527) as used by the shoot loop (source/Main.cpp:1170-1183).
// The library is compiled with -fmad=false and IEEE division / square root, so
// each expression rounds exactly as the reference's float code does; the
// projection matrix (which needs tan) is computed once on the host.
#pragma once
#include <cuda_runtime.h>

namespace rad {

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 neg(f3 a) { return mk(-a.x, -a.y, -a.z); }
// Vector3::v_Cross / Vector3::Cross (source/Vector.h:534-545): note the operand order.
__device__ __forceinline__ f3 vcross(f3 a, f3 b) {
    return mk(b.y * a.z - b.z * a.y, b.z * a.x - b.x * a.z, b.x * a.y - b.y * a.x);
}
// Vector3::Normalize (source/Vector.h:389-399).
__device__ __forceinline__ f3 normalize(f3 v) {
    float t = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    if (t != 0) {
        t = 1 / t;
        v.x *= t;
        v.y *= t;
        v.z *= t;
    }
    return v;
}

// r = a*b in Matrix4f::ProductOf order; m[col*4+row].
__device__ __forceinline__ void mat_mul(const float* a, const float* b, float* r) {
    float t[16];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            t[i * 4 + j] = a[0 * 4 + j] * b[i * 4 + 0] + a[1 * 4 + j] * b[i * 4 + 1] + a[2 * 4 + j] * b[i * 4 + 2] +
                           a[3 * 4 + j] * b[i * 4 + 3];
#pragma unroll
    for (int i = 0; i < 16; i++) r[i] = t[i];
}

__device__ __forceinline__ void mat_identity(float* m) {
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) m[i * 4 + j] = (float)(i == j);
}

// Center, (un-normalised) normal and up of the quad q[12].
__device__ __forceinline__ void patch_frame(const float* q, f3& c, f3& n, f3& u) {
    f3 v1 = mk(q[0], q[1], q[2]), v2 = mk(q[3], q[4], q[5]), v3 = mk(q[6], q[7], q[8]), v4 = mk(q[9], q[10], q[11]);
    c = mk((v1.x + v2.x + v3.x + v4.x) / 4.0f, (v1.y + v2.y + v3.y + v4.y) / 4.0f,
           (v1.z + v2.z + v3.z + v4.z) / 4.0f);
    n = vcross(sub(v2, v1), sub(v4, v1));
    u = sub(v4, v1);
}

// MVP of face loop index `face` (0 UP, 1 DOWN, 2 LEFT, 3 RIGHT, 4 FRONT;
// p_patchlook_perm of source/Main.h:210) for quad q; proj = the host's projection.
__device__ __forceinline__ void face_mvp(const float* q, int face, const float* proj, float* out) {
    f3 eye, normal, pup;
    patch_frame(q, eye, normal, pup);
    f3 target, up;
    switch (face) {
        case 0: target = pup; up = neg(normal); break;
        case 1: target = neg(pup); up = normal; break;
        case 2: target = neg(vcross(normal, pup)); up = pup; break;
        case 3: target = vcross(normal, pup); up = pup; break;
        default: target = normal; up = pup; break;
    }
    f3 dir = normalize(sub(add(target, eye), eye));
    f3 right = normalize(vcross(dir, up));
    f3 u2 = vcross(right, dir);
    float la[16];
    la[0] = right.x; la[4] = right.y; la[8] = right.z;
    la[1] = u2.x; la[5] = u2.y; la[9] = u2.z;
    la[2] = -dir.x; la[6] = -dir.y; la[10] = -dir.z;
    la[3] = 0; la[7] = 0; la[11] = 0;
    la[12] = 0; la[13] = 0; la[14] = 0;
    la[15] = 1;
    float tr[16];
    mat_identity(tr);
    tr[12] = -eye.x; tr[13] = -eye.y; tr[14] = -eye.z;
    mat_mul(la, tr, la);
    float mv[16];
    mat_identity(mv);
    mat_mul(mv, la, mv);
    mat_mul(proj, mv, out);
}

}  // namespace rad
