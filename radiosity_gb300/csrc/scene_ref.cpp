// The reference scene: ModelContainer::load (source/ModelContainer.cpp:89-110)
// = PrimitiveModel ROOM, ROOMCLOSURE, CUBE, BLOCK (source/PrimitiveModel.cpp:4-213),
// each subdivided once by Model::subdivide / Patch::divide
// (source/Model.cpp:49-82, source/Patch.cpp:47-125) and flattened by
// ModelContainer::updateData (source/ModelContainer.cpp:135-209).
//
// The corner coordinates below are the reference scene's data (the classic
// Cornell box measurements in metres); they have to be identical for the solve
// to be comparable, so they are carried over as data.  The subdivision follows
// the reference's float/double expression order so the patch corners are
// bit-identical (pinned against the compiled reference in the test suite).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "radiosity.h"

namespace {

struct V3 {
    float x, y, z;
};
V3 v(float x, float y, float z) { return V3{x, y, z}; }
V3 operator-(V3 a, V3 b) { return v(a.x - b.x, a.y - b.y, a.z - b.z); }
V3 operator+(V3 a, V3 b) { return v(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 operator*(V3 a, float t) { return v(a.x * t, a.y * t, a.z * t); }
V3 operator/(V3 a, float t) {  // Vector3::operator/(T): multiplies by 1/t
    t = 1 / t;
    return v(a.x * t, a.y * t, a.z * t);
}
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float length(V3 a) { return (float)std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

struct Quad {
    V3 c[4];
    V3 color, illum, rad;
};

// x y z of 4 corners per quad, 5 quads per part (source/PrimitiveModel.cpp:132-245).
const float kRoom[60] = {0.0f, 0.0f, 5.592f, 5.496f, 0.0f, 5.592f, 5.560f, 5.488f, 5.592f, 0.0f, 5.488f, 5.592f,
                         0.0f, 5.488f, 0.0f, 0.0f, 5.488f, 5.592f, 5.560f, 5.488f, 5.592f, 5.560f, 5.488f, 0.0f,
                         0.0f, 0.0f, 0.0f, 5.528f, 0.0f, 0.0f, 5.496f, 0.0f, 5.592f, 0.0f, 0.0f, 5.592f,
                         0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 5.592f, 0.0f, 5.488f, 5.593f, 0.0f, 5.488f, 0.0f,
                         5.496f, 0.0f, 5.592f, 5.528f, 0.0f, 0.0f, 5.560f, 5.488f, 0.0f, 5.560f, 5.488f, 5.592f};
const float kRoomColors[15] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 1, 0};
const float kClosure[12] = {5.528f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 5.488f, 0.0f, 5.560f, 5.488f, 0.0f};
const float kCube[60] = {1.3f, 1.65f, 0.65f, 2.9f, 1.65f, 1.14f, 2.4f, 1.65f, 2.72f, 0.82f, 1.65f, 2.25f,
                         2.9f, 0.0f, 1.14f, 2.4f, 0.0f, 2.72f, 2.4f, 1.65f, 2.72f, 2.9f, 1.65f, 1.14f,
                         1.3f, 0.0f, 0.65f, 2.9f, 0.0f, 1.14f, 2.9f, 1.65f, 1.14f, 1.3f, 1.65f, 0.65f,
                         0.82f, 0.0f, 2.25f, 1.3f, 0.0f, 0.65f, 1.3f, 1.65f, 0.65f, 0.82f, 1.65f, 2.25f,
                         2.4f, 0.0f, 2.72f, 0.82f, 0.0f, 2.25f, 0.82f, 1.65f, 2.25f, 2.4f, 1.65f, 2.72f};
const float kBlock[60] = {4.23f, 3.3f, 2.47f, 4.72f, 3.3f, 4.06f, 3.14f, 3.3f, 4.56f, 2.65f, 3.3f, 2.96f,
                          4.23f, 0.0f, 2.47f, 4.72f, 0.0f, 4.06f, 4.72f, 3.3f, 4.06f, 4.23f, 3.3f, 2.47f,
                          4.72f, 0.0f, 4.06f, 3.14f, 0.0f, 4.56f, 3.14f, 3.3f, 4.56f, 4.72f, 3.3f, 4.06f,
                          3.14f, 0.0f, 4.56f, 2.65f, 0.0f, 2.96f, 2.65f, 3.3f, 2.96f, 3.14f, 3.3f, 4.56f,
                          2.65f, 0.0f, 2.96f, 4.23f, 0.0f, 2.47f, 4.23f, 3.3f, 2.47f, 2.65f, 3.3f, 2.96f};

Quad quad_from(const float* p, V3 color) {
    Quad q;
    for (int k = 0; k < 4; k++) q.c[k] = v(p[3 * k], p[3 * k + 1], p[3 * k + 2]);
    q.color = color;
    q.illum = v(0, 0, 0);
    q.rad = v(0, 0, 0);
    return q;
}

// Patch::divide + Model::subdivide for one quad, appended to out.
void subdivide(const Quad& p, double area, std::vector<Quad>& out) {
    V3 A = p.c[0], B = p.c[1], C = p.c[2], D = p.c[3];
    V3 u1 = A - C, u2 = B - D;
    double phi = std::acos(dot(u1, u2) / (length(u1) * length(u2)));
    double S = 0.5f * length(u1) * length(u2) * std::sin(phi);
    if (S <= (area * 1.01)) {
        out.push_back(p);
        return;
    }
    double a = std::sqrt(area);
    unsigned kx = (unsigned)(std::ceil(length(B - A) / a));
    unsigned ky = (unsigned)(std::ceil(length(C - B) / a));
    V3 pCD = (C - D) / float(kx);
    V3 pAB = (B - A) / float(kx);
    for (unsigned i = 0; i < kx * ky; i++) {
        unsigned col = i % kx, row = i / kx;
        V3 bCD = pCD * float(col) + D, bAB = pAB * float(col) + A;
        V3 nA = bAB + ((bCD - bAB) / float(ky)) * float(row);
        V3 bCD1 = pCD * float(col + 1) + D, bAB1 = pAB * float(col + 1) + A;
        V3 nB = bAB1 + ((bCD1 - bAB1) / float(ky)) * float(row);
        V3 nC = bAB1 + ((bCD1 - bAB1) / float(ky)) * float(row + 1);
        V3 nD = bAB + ((bCD - bAB) / float(ky)) * float(row + 1);
        Quad q;
        q.c[0] = nA; q.c[1] = nB; q.c[2] = nC; q.c[3] = nD;
        q.color = p.color;
        q.illum = p.illum;
        q.rad = p.rad;
        out.push_back(q);
    }
}

std::vector<Quad> reference_scene(double area) {
    std::vector<std::vector<Quad>> models(4);
    for (int i = 0; i < 60; i += 12)
        models[0].push_back(quad_from(kRoom + i, v(kRoomColors[i / 4], kRoomColors[i / 4 + 1], kRoomColors[i / 4 + 2])));
    {  // the light (source/PrimitiveModel.cpp:21-29)
        Quad l;
        l.c[0] = v(3.430f, 5.485f, 2.270f);
        l.c[1] = v(2.130f, 5.485f, 2.270f);
        l.c[2] = v(2.130f, 5.485f, 3.320f);
        l.c[3] = v(3.430f, 5.485f, 3.320f);
        l.color = v(1.0f, 1.0f, 1.0f);
        l.illum = v(1.0f, 1.0f, 1.0f);
        l.rad = l.illum * 100;
        models[0].push_back(l);
    }
    models[1].push_back(quad_from(kClosure, v(1, 1, 1)));
    for (int i = 0; i < 60; i += 12) models[2].push_back(quad_from(kCube + i, v(1, 1, 1)));
    for (int i = 0; i < 60; i += 12) models[3].push_back(quad_from(kBlock + i, v(1, 1, 1)));
    std::vector<Quad> all;
    for (auto& m : models) {
        if (area > 0) {
            std::vector<Quad> sub;
            for (auto& q : m) subdivide(q, area, sub);
            all.insert(all.end(), sub.begin(), sub.end());
        } else {
            all.insert(all.end(), m.begin(), m.end());
        }
    }
    return all;
}

}  // namespace

extern "C" int rad_scene_reference(double max_patch_area, uint32_t capacity, uint32_t* n, float* vertices,
                                   int32_t* indices, float* color, float* radiosity, float* illumination) {
    if (!n) return RAD_E_INVALID;
    std::vector<Quad> s = reference_scene(max_patch_area);
    *n = (uint32_t)s.size();
    if (!vertices && !indices && !color && !radiosity && !illumination) return RAD_OK;
    if (capacity < s.size()) return RAD_E_INVALID;
    for (size_t i = 0; i < s.size(); i++) {
        const Quad& q = s[i];
        if (vertices)
            for (int k = 0; k < 4; k++) {
                vertices[12 * i + 3 * k] = q.c[k].x;
                vertices[12 * i + 3 * k + 1] = q.c[k].y;
                vertices[12 * i + 3 * k + 2] = q.c[k].z;
            }
        if (indices) {
            const int32_t b = (int32_t)(4 * i);
            const int32_t pat[6] = {b, b + 1, b + 2, b, b + 2, b + 3};
            std::memcpy(indices + 6 * i, pat, sizeof(pat));
        }
        const V3* src[3] = {&q.color, &q.rad, &q.illum};
        float* dst[3] = {color, radiosity, illumination};
        for (int a = 0; a < 3; a++)
            if (dst[a]) {
                dst[a][3 * i] = src[a]->x;
                dst[a][3 * i + 1] = src[a]->y;
                dst[a][3 * i + 2] = src[a]->z;
            }
    }
    return RAD_OK;
}
