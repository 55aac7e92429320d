// Host-side scene builders and scene files of the reference:
//  * the reference scene: ModelContainer::load (source/ModelContainer.cpp:35-56)
//    = PrimitiveModel ROOM, ROOMCLOSURE, CUBE, BLOCK (source/PrimitiveModel.cpp:4-213),
//    each subdivided once by Model::subdivide / Patch::divide
//    (source/Model.cpp:27-60, source/Patch.cpp:47-222) and flattened by
//    ModelContainer::updateData (source/ModelContainer.cpp:81-155);
//  * the 8 display neighbours of every patch (source/Patch.cpp:128-219; a patch
//    that was not divided is its own neighbour, source/Model.cpp:38-46);
//  * Wavefront OBJ quads (WaveFrontModel::parse, source/WaveFrontModel.cpp:15-143);
//  * the .rr scene files of SaveToFile / LoadFromFile (source/Main.cpp:1460-1647,
//    source/LoadingModel.cpp:4-17).
//
// The corner coordinates below are the reference scene's data (the classic
// Cornell box measurements in metres); they have to be identical for the solve
// to be comparable, so they are carried over as data.  The subdivision follows
// the reference's float/double expression order so the patch corners are
// bit-identical (pinned against the compiled reference in the test suite).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
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
    uint32_t nb[8];  // scene-global indices of the display neighbours (source/Patch.h:50)
};
void self_neighbours(Quad& q, uint32_t self) {
    for (int j = 0; j < 8; j++) q.nb[j] = self;
}

// x y z of 4 corners per quad, 5 quads per part (source/PrimitiveModel.cpp:4-213).
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
        self_neighbours(out.back(), (uint32_t)(out.size() - 1));
        return;
    }
    double a = std::sqrt(area);
    unsigned kx = (unsigned)(std::ceil(length(B - A) / a));
    unsigned ky = (unsigned)(std::ceil(length(C - B) / a));
    V3 pCD = (C - D) / float(kx);
    V3 pAB = (B - A) / float(kx);
    const uint32_t base = (uint32_t)out.size();
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
        // neighbours in the child grid, numbered from the upper left corner clockwise,
        // with the reference's fall-backs at the grid border (source/Patch.cpp:128-219)
        const uint32_t self = base + i;
        auto at = [&](unsigned r, unsigned c) { return base + r * kx + c; };
        const bool top = row + 1 >= ky, bottom = row == 0, left = col == 0, right = col + 1 >= kx;
        q.nb[0] = top ? (!left ? at(row, col - 1) : self) : (left ? at(row + 1, col) : at(row + 1, col - 1));
        q.nb[1] = top ? self : at(row + 1, col);
        q.nb[2] = top ? (!right ? at(row, col + 1) : self) : (right ? at(row + 1, col) : at(row + 1, col + 1));
        q.nb[3] = right ? self : at(row, col + 1);
        q.nb[4] = bottom ? (!right ? at(row, col + 1) : self) : (right ? at(row - 1, col) : at(row - 1, col + 1));
        q.nb[5] = bottom ? self : at(row - 1, col);
        q.nb[6] = bottom ? (!left ? at(row, col - 1) : self) : (left ? at(row - 1, col) : at(row - 1, col - 1));
        q.nb[7] = left ? self : at(row, col - 1);
        out.push_back(q);
    }
}

// Model::getPatches(area) + ModelContainer::updateData for a list of models: each model
// is subdivided when area > 0, patches are concatenated in model order and their
// neighbour indices shifted to scene-global numbering.
std::vector<Quad> flatten(const std::vector<std::vector<Quad>>& models, double area) {
    std::vector<Quad> all;
    for (const auto& m : models) {
        std::vector<Quad> sub;
        if (area > 0) {
            for (const auto& q : m) subdivide(q, area, sub);
        } else {
            sub = m;
            for (size_t i = 0; i < sub.size(); i++) self_neighbours(sub[i], (uint32_t)i);
        }
        const uint32_t off = (uint32_t)all.size();
        for (auto& q : sub)
            for (int j = 0; j < 8; j++) q.nb[j] += off;
        all.insert(all.end(), sub.begin(), sub.end());
    }
    return all;
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
    return flatten(models, area);
}

// WaveFrontModel::parse (source/WaveFrontModel.cpp:15-143) on an in-memory file: "v x y z"
// lines give vertices scaled by 1/1000 (a 4th coordinate is ignored), "f a b c [d]" lines
// give quads from 1-based vertex numbers (anything after a '/' is ignored); a triangle
// repeats its last vertex, faces with another vertex count and faces naming a missing
// vertex are skipped.  Patches start black with no energy (source/Patch.cpp:8-13).
// Returns false on a vertex line with fewer than 3 coordinates (the reference's error).
bool parse_obj(const char* text, size_t len, std::vector<Quad>& quads) {
    std::vector<V3> verts;
    size_t pos = 0;
    while (pos < len) {
        size_t end = pos;
        while (end < len && text[end] != '\n') end++;
        std::string line(text + pos, end - pos);
        pos = end + 1;
        if (line.compare(0, 2, "v ") == 0) {
            std::vector<float> pts;
            const char* c = line.c_str() + 2;
            for (;;) {  // istream >> float: white space, then [+-]digits[.digits][e[+-]digits]
                while (*c == ' ' || *c == '\t' || *c == '\r' || *c == '\v' || *c == '\f') c++;
                const char* e = c;
                if (*e == '+' || *e == '-') e++;
                bool digits = false;
                while (*e >= '0' && *e <= '9') e++, digits = true;
                if (*e == '.') {
                    e++;
                    while (*e >= '0' && *e <= '9') e++, digits = true;
                }
                if (!digits) break;
                if (*e == 'e' || *e == 'E') {
                    const char* x = e + 1;
                    if (*x == '+' || *x == '-') x++;
                    if (*x >= '0' && *x <= '9') {
                        while (*x >= '0' && *x <= '9') x++;
                        e = x;
                    }
                }
                pts.push_back(std::strtof(std::string(c, e).c_str(), nullptr));
                c = e;
            }
            if (pts.size() < 3) return false;
            verts.push_back(v(pts[0] / 1000, pts[1] / 1000, pts[2] / 1000));
        } else if (line.compare(0, 2, "f ") == 0) {
            std::string rest = line.substr(2);
            std::vector<long long> fv;
            while (!rest.empty() && fv.size() <= 4) {
                const size_t sp = rest.find_first_of(' ');
                const std::string tok = rest.substr(0, sp);
                // istream >> int: optional white space and sign, then digits
                const char* c = tok.c_str();
                while (*c == ' ' || *c == '\t' || *c == '\r' || *c == '\v' || *c == '\f') c++;
                char* e = nullptr;
                const long long k = std::strtoll(c, &e, 10);
                if (e != c && k >= -2147483648LL && k <= 2147483647LL) fv.push_back(k - 1);
                if (sp == std::string::npos) rest.clear();
                else rest.erase(0, sp + 1);
            }
            if (fv.size() == 3) fv.push_back(fv.back());
            if (fv.size() != 4) continue;
            bool ok = true;
            for (long long k : fv) ok = ok && k >= 0 && (unsigned long long)k < verts.size();
            if (!ok) continue;  // vector::at out_of_range: the face is skipped
            Quad q;
            for (int k = 0; k < 4; k++) q.c[k] = verts[(size_t)fv[k]];
            q.color = v(0, 0, 0);
            q.illum = v(0, 0, 0);
            q.rad = v(0, 0, 0);
            quads.push_back(q);
        }
    }
    return true;
}

// .rr patch record: the reference's Patch object as fwrite'd by SaveToFile.  Field order
// radiosity, illumination, relativeNeighbours[8], neighbours[8] (pointers, written NULL),
// vec1..vec4, color; 148 bytes with 4-byte pointers (32-bit build), 184 with 8-byte
// pointers (64-bit build, 4 bytes of tail padding).  The file starts with the patch count
// as a 32-bit unsigned long.
size_t rr_record(uint32_t ptr) { return ptr == 4 ? 148 : 184; }
size_t rr_vec_offset(uint32_t ptr) { return 24 + 32 + 8 * (size_t)ptr; }

void put3(unsigned char* d, V3 a) {
    const float f[3] = {a.x, a.y, a.z};
    std::memcpy(d, f, 12);
}
V3 get3(const unsigned char* d) {
    float f[3];
    std::memcpy(f, d, 12);
    return v(f[0], f[1], f[2]);
}

int export_scene(const std::vector<Quad>& s, uint32_t capacity, uint32_t* n, float* vertices, int32_t* indices,
                 float* color, float* radiosity, float* illumination, uint32_t* neighbours) {
    *n = (uint32_t)s.size();
    if (!vertices && !indices && !color && !radiosity && !illumination && !neighbours) return RAD_OK;
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
        if (neighbours) std::memcpy(neighbours + 8 * i, q.nb, sizeof(q.nb));
    }
    return RAD_OK;
}

}  // namespace

extern "C" int rad_scene_reference(double max_patch_area, uint32_t capacity, uint32_t* n, float* vertices,
                                   int32_t* indices, float* color, float* radiosity, float* illumination) {
    if (!n) return RAD_E_INVALID;
    return export_scene(reference_scene(max_patch_area), capacity, n, vertices, indices, color, radiosity, illumination,
                        nullptr);
}

extern "C" int rad_scene_reference_neighbours(double max_patch_area, uint32_t capacity, uint32_t* n,
                                              uint32_t* neighbours) {
    if (!n) return RAD_E_INVALID;
    return export_scene(reference_scene(max_patch_area), capacity, n, nullptr, nullptr, nullptr, nullptr, nullptr,
                        neighbours);
}

extern "C" int rad_scene_obj(const char* text, uint64_t length, double max_patch_area, uint32_t capacity, uint32_t* n,
                             float* vertices, int32_t* indices, float* color, float* radiosity, float* illumination,
                             uint32_t* neighbours) {
    if (!n || (!text && length)) return RAD_E_INVALID;
    std::vector<std::vector<Quad>> models(1);
    if (!parse_obj(text, (size_t)length, models[0])) return RAD_E_INVALID;
    return export_scene(flatten(models, max_patch_area), capacity, n, vertices, indices, color, radiosity,
                        illumination, neighbours);
}

extern "C" int rad_rr_size(uint32_t n, uint32_t pointer_bytes, uint64_t* bytes) {
    if (!bytes || (pointer_bytes != 4 && pointer_bytes != 8)) return RAD_E_INVALID;
    *bytes = 4 + (uint64_t)n * rr_record(pointer_bytes);
    return RAD_OK;
}

extern "C" int rad_rr_write(uint32_t n, const float* vertices, const float* color, const float* radiosity,
                            const float* illumination, const uint32_t* neighbours, uint32_t pointer_bytes, void* out,
                            uint64_t capacity) {
    uint64_t need = 0;
    if (rad_rr_size(n, pointer_bytes, &need) != RAD_OK || !out || capacity < need) return RAD_E_INVALID;
    if (n && (!vertices || !color || !radiosity || !illumination)) return RAD_E_INVALID;
    unsigned char* d = static_cast<unsigned char*>(out);
    std::memset(d, 0, (size_t)need);
    std::memcpy(d, &n, 4);
    const size_t rec = rr_record(pointer_bytes), vo = rr_vec_offset(pointer_bytes);
    for (uint32_t i = 0; i < n; i++) {
        unsigned char* r = d + 4 + (size_t)i * rec;
        put3(r, v(radiosity[3 * i], radiosity[3 * i + 1], radiosity[3 * i + 2]));
        put3(r + 12, v(illumination[3 * i], illumination[3 * i + 1], illumination[3 * i + 2]));
        for (int j = 0; j < 8; j++) {
            const uint32_t nb = neighbours ? neighbours[8 * (size_t)i + j] : i;
            if (nb >= n) return RAD_E_INVALID;
            std::memcpy(r + 24 + 4 * j, &nb, 4);
        }
        for (int k = 0; k < 4; k++)
            put3(r + vo + 12 * k, v(vertices[12 * (size_t)i + 3 * k], vertices[12 * (size_t)i + 3 * k + 1],
                                    vertices[12 * (size_t)i + 3 * k + 2]));
        put3(r + vo + 48, v(color[3 * i], color[3 * i + 1], color[3 * i + 2]));
    }
    return RAD_OK;
}

extern "C" int rad_rr_read(const void* data, uint64_t length, uint32_t capacity, uint32_t* n, float* vertices,
                           int32_t* indices, float* color, float* radiosity, float* illumination,
                           uint32_t* neighbours, uint32_t* pointer_bytes) {
    if (!n || !data || length < 4) return RAD_E_INVALID;
    const unsigned char* d = static_cast<const unsigned char*>(data);
    uint32_t count;
    std::memcpy(&count, d, 4);
    uint32_t ptr = 0;
    if ((uint64_t)count * 148 + 4 == length) ptr = 4;
    else if ((uint64_t)count * 184 + 4 == length) ptr = 8;
    else return RAD_E_INVALID;  // neither a 32-bit nor a 64-bit build's file of `count` patches
    if (pointer_bytes) *pointer_bytes = ptr;
    const size_t rec = rr_record(ptr), vo = rr_vec_offset(ptr);
    std::vector<Quad> s(count);
    for (uint32_t i = 0; i < count; i++) {
        const unsigned char* r = d + 4 + (size_t)i * rec;
        Quad& q = s[i];
        q.rad = get3(r);
        q.illum = get3(r + 12);
        for (int j = 0; j < 8; j++) {
            std::memcpy(&q.nb[j], r + 24 + 4 * j, 4);
            if (q.nb[j] >= count) return RAD_E_INVALID;  // LoadingModel's patches->at() would throw
        }
        for (int k = 0; k < 4; k++) q.c[k] = get3(r + vo + 12 * k);
        q.color = get3(r + vo + 48);
    }
    return export_scene(s, capacity, n, vertices, indices, color, radiosity, illumination, neighbours);
}
