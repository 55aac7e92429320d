/* oracle.c - CPU restatement of the reference's hemicube shoot loop.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h for who may load it and what is pinned).
 * Compiled with -ffp-contract=off so every float expression rounds exactly as
 * written; the product's CUDA kernels follow the same operation order.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.1415926535897932384626433832795028841931f /* source/FormFactors.cpp:3 */
#define ORC_GUARD 1024.0f
#define ORC_REFLECTIVITY 0.3f /* source/Patch.h:13 */

/* ------------------------------------------------------------------------- */
/* Delta form factors: source/FormFactors.cpp:23-67 and :280-314               */
/* ------------------------------------------------------------------------- */
static void ff_front_side(int n, float* front, float* side) {
    float hpw = (1.0f / n);
    float pix = (2.0f / n);
    pix *= pix;
    for (int x = 0; x < n; x++)
        for (int y = 0; y < n; y++) {
            float dx = ((x - n / 2) / (n / 2.0f)) + hpw;
            float dy = ((y - n / 2) / (n / 2.0f)) + hpw;
            float f = (dx * dx + dy * dy + 1);
            f *= f * ORC_PI;
            front[x + y * n] = pix / f;
        }
    for (int x = 0; x < n; x++)
        for (int y = 0; y < n / 2; y++) {
            float dx = (x - n / 2) / (n / 2.0f) + hpw;
            float dy = (n / 2 - 1 - y) / (n / 2.0f) + hpw;
            float f = (dx * dx + dy * dy + 1);
            f *= f * ORC_PI;
            side[x + y * n] = (pix * (dy + hpw)) / f;
        }
}

int orc_ff_table(uint32_t W, float* out) {
    if (W < 2 || (W & 1u)) return -1;
    float* front = (float*)malloc(sizeof(float) * W * W);
    float* side = (float*)malloc(sizeof(float) * W * W / 2);
    ff_front_side((int)W, front, side);
    const uint32_t H = W, TW = 2 * W, TH = (uint32_t)(H * 1.5), RES = TW * TH;
    for (uint32_t i = 0; i < RES; i++) {
        uint32_t x = i % TW, y = i / TW;
        if (x >= W / 2 && x < W * 1.5 && y < H)
            out[i] = front[y * W + (x - W / 2)];
        else if (x < W / 2 && y < H)
            out[i] = side[(H / 2 - x) * W - y - 1];
        else if (x >= W * 1.5 && y < H)
            out[i] = side[(x - (uint32_t)(W * 1.5)) * W + y];
        else if (x < W && y >= H)
            out[i] = side[(y - H) * W + x];
        else if (x >= W && y >= H)
            out[i] = side[((H / 2 - 1) - (y - H)) * W + (x - W)];
    }
    free(front);
    free(side);
    return 0;
}

float orc_ff_sum(uint32_t W) {
    int n = (int)W;
    float* front = (float*)malloc(sizeof(float) * W * W);
    float* side = (float*)malloc(sizeof(float) * W * W / 2);
    ff_front_side(n, front, side);
    float s = 0;
    for (int y = 0; y < n; y++)
        for (int x = 0; x < n / 2; x++) s += side[y + x * n];
    s *= 4;
    for (int x = 0; x < n; x++)
        for (int y = 0; y < n; y++) s += front[x + y * n];
    free(front);
    free(side);
    return s;
}

/* ------------------------------------------------------------------------- */
/* Face rectangles: source/Main.cpp:316-389                                   */
/* ------------------------------------------------------------------------- */
void orc_face_rects(uint32_t W, uint32_t hi, int face, int vp[4], int sc[4]) {
    int w = (int)W, h = (int)W, off = (int)(W * 1.5 * hi);
    vp[2] = w;
    vp[3] = h;
    switch (face) {
        case 0: vp[0] = 0; vp[1] = h + off; break;
        case 1: vp[0] = w; vp[1] = h / 2 + off; break;
        case 2: vp[0] = -1 * (int)(W / 2); vp[1] = off; break;
        case 3: vp[0] = (int)(W * 1.5); vp[1] = off; break;
        default: vp[0] = w / 2; vp[1] = off; break;
    }
    if (face == 0 || face == 1) {
        sc[1] = h + off;
        sc[3] = h / 2;
    } else {
        sc[1] = off;
        sc[3] = h;
    }
    sc[2] = (face == 2 || face == 3) ? w / 2 : w;
    switch (face) {
        case 0: case 2: sc[0] = 0; break;
        case 1: sc[0] = w; break;
        case 3: sc[0] = (int)(W * 1.5); break;
        default: sc[0] = w / 2; break;
    }
}

/* ------------------------------------------------------------------------- */
/* Cameras: Vector3 ops of source/Vector.h:351-545, Matrix4f of Vector.cpp     */
/* ------------------------------------------------------------------------- */
typedef struct { float x, y, z; } v3;

static v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 neg3(v3 a) { return mk3(-a.x, -a.y, -a.z); }
/* a.v_Cross(b) and a.Cross(b): (b.y*a.z - b.z*a.y, b.z*a.x - b.x*a.z, b.x*a.y - b.y*a.x) */
static v3 vcross(v3 a, v3 b) {
    return mk3(b.y * a.z - b.z * a.y, b.z * a.x - b.x * a.z, b.x * a.y - b.y * a.x);
}
static v3 normalize3(v3 v) {
    float t = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    if (t != 0) {
        t = 1 / t;
        v.x *= t;
        v.y *= t;
        v.z *= t;
    }
    return v;
}

/* m[col*4+row]; r = a*b with the summation order of Matrix4f::ProductOf. */
static void matmul(const float* a, const float* b, float* r) {
    float t[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            t[i * 4 + j] = a[0 * 4 + j] * b[i * 4 + 0] + a[1 * 4 + j] * b[i * 4 + 1] +
                           a[2 * 4 + j] * b[i * 4 + 2] + a[3 * 4 + j] * b[i * 4 + 3];
    memcpy(r, t, sizeof(t));
}
static void identity(float* m) {
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++) m[i * 4 + j] = (float)(i == j);
}

void orc_patch_frame(const float* q, float* out) {
    v3 v1 = mk3(q[0], q[1], q[2]), v2 = mk3(q[3], q[4], q[5]), v3_ = mk3(q[6], q[7], q[8]),
       v4 = mk3(q[9], q[10], q[11]);
    out[0] = (v1.x + v2.x + v3_.x + v4.x) / 4.0f;
    out[1] = (v1.y + v2.y + v3_.y + v4.y) / 4.0f;
    out[2] = (v1.z + v2.z + v3_.z + v4.z) / 4.0f;
    v3 n = vcross(sub3(v2, v1), sub3(v4, v1));
    out[3] = n.x; out[4] = n.y; out[5] = n.z;
    v3 u = sub3(v4, v1);
    out[6] = u.x; out[7] = u.y; out[8] = u.z;
}

void orc_face_mvp(const float* q, int face, float* out) {
    float fr[9];
    orc_patch_frame(q, fr);
    v3 eye = mk3(fr[0], fr[1], fr[2]), normal = mk3(fr[3], fr[4], fr[5]), pup = mk3(fr[6], fr[7], fr[8]);
    v3 target, up;
    switch (face) { /* loop index -> PatchLook via source/Main.h:210 */
        case ORC_FACE_UP: target = pup; up = neg3(normal); break;
        case ORC_FACE_DOWN: target = neg3(pup); up = normal; break;
        case ORC_FACE_LEFT: target = neg3(vcross(normal, pup)); up = pup; break;
        case ORC_FACE_RIGHT: target = vcross(normal, pup); up = pup; break;
        default: target = normal; up = pup; break;
    }
    /* LookAt(m, eye, target + eye, up) */
    v3 dir = sub3(add3(target, eye), eye);
    dir = normalize3(dir);
    v3 right = normalize3(vcross(dir, up));
    v3 u2 = vcross(right, dir);
    float la[16];
    la[0 * 4 + 0] = right.x; la[1 * 4 + 0] = right.y; la[2 * 4 + 0] = right.z;
    la[0 * 4 + 1] = u2.x; la[1 * 4 + 1] = u2.y; la[2 * 4 + 1] = u2.z;
    la[0 * 4 + 2] = -dir.x; la[1 * 4 + 2] = -dir.y; la[2 * 4 + 2] = -dir.z;
    for (int i = 0; i < 3; i++) {
        la[i * 4 + 3] = 0;
        la[3 * 4 + i] = 0;
    }
    la[15] = 1;
    float tr[16];
    identity(tr);
    tr[12] = -eye.x; tr[13] = -eye.y; tr[14] = -eye.z;
    matmul(la, tr, la);
    float mv[16];
    identity(mv);
    matmul(mv, la, mv);
    /* Perspective(90, 1, 0.01, 1000) -> Frustum(-fw, fw, -fh, fh, n, f) */
    float fov = 90, aspect = 1.0f, n = 0.01f, f = 1000;
    float fh = (float)(tanf(fov * ORC_PI / 180 * .5f)) * n;
    float fw = fh * aspect;
    float l = -fw, r = fw, b = -fh, t = fh;
    float p[16];
    p[0] = 2 * n / (r - l); p[4] = 0; p[8] = (r + l) / (r - l); p[12] = 0;
    p[1] = 0; p[5] = 2 * n / (t - b); p[9] = (t + b) / (t - b); p[13] = 0;
    p[2] = 0; p[6] = 0; p[10] = -(f + n) / (f - n); p[14] = -2 * f * n / (f - n);
    p[3] = 0; p[7] = 0; p[11] = -1; p[15] = 0;
    matmul(p, mv, out);
}

/* ------------------------------------------------------------------------- */
/* Raster contract (see oracle.h)                                             */
/* ------------------------------------------------------------------------- */
typedef struct { float x, y, z, w; } v4;

static float plane_dist(int plane, v4 v) {
    switch (plane) {
        case 0: return v.z + v.w;
        case 1: return v.w - v.z;
        case 2: return ORC_GUARD * v.w - v.x;
        case 3: return ORC_GUARD * v.w + v.x;
        case 4: return ORC_GUARD * v.w - v.y;
        default: return ORC_GUARD * v.w + v.y;
    }
}

/* Sutherland-Hodgman over the six planes; returns vertex count (<= 9). */
static int clip_polygon(v4* poly, int n) {
    v4 tmp[12];
    for (int pl = 0; pl < 6 && n > 0; pl++) {
        float d[12];
        int all_in = 1;
        for (int i = 0; i < n; i++) {
            d[i] = plane_dist(pl, poly[i]);
            if (!(d[i] >= 0)) all_in = 0;
        }
        if (all_in) continue;
        int m = 0;
        for (int i = 0; i < n; i++) {
            int j = (i + 1 == n) ? 0 : i + 1;
            v4 a = poly[i], b = poly[j];
            int ain = d[i] >= 0, bin = d[j] >= 0;
            if (ain) tmp[m++] = a;
            if (ain != bin) {
                float t = d[i] / (d[i] - d[j]);
                v4 c;
                c.x = a.x + t * (b.x - a.x);
                c.y = a.y + t * (b.y - a.y);
                c.z = a.z + t * (b.z - a.z);
                c.w = a.w + t * (b.w - a.w);
                tmp[m++] = c;
            }
        }
        n = m;
        memcpy(poly, tmp, sizeof(v4) * (size_t)m);
    }
    return n;
}

static int64_t floordiv256(int64_t a) { return (a >= 0) ? a / 256 : -((-a + 255) / 256); }

static uint32_t depth_ordinal(float d) {
    if (!(d > 0)) return 0x7F800000u;
    uint32_t b;
    memcpy(&b, &d, 4);
    if (b >= 0x7F800000u) return 0;
    return 0x7F800000u - b;
}

typedef struct {
    int32_t X, Y;
    float D;
} sv;

static void raster_triangle(sv a, sv b, sv c, uint32_t id, const int sc[4], uint32_t TW, uint64_t* zbuf) {
    int64_t area2 = ((int64_t)b.X - a.X) * ((int64_t)c.Y - a.Y) - ((int64_t)c.X - a.X) * ((int64_t)b.Y - a.Y);
    if (area2 <= 0) return;
    int32_t xmin = a.X, xmax = a.X, ymin = a.Y, ymax = a.Y;
    if (b.X < xmin) xmin = b.X;
    if (c.X < xmin) xmin = c.X;
    if (b.X > xmax) xmax = b.X;
    if (c.X > xmax) xmax = c.X;
    if (b.Y < ymin) ymin = b.Y;
    if (c.Y < ymin) ymin = c.Y;
    if (b.Y > ymax) ymax = b.Y;
    if (c.Y > ymax) ymax = c.Y;
    int64_t px0 = floordiv256((int64_t)xmin - 128 + 255), px1 = floordiv256((int64_t)xmax - 128);
    int64_t py0 = floordiv256((int64_t)ymin - 128 + 255), py1 = floordiv256((int64_t)ymax - 128);
    if (px0 < sc[0]) px0 = sc[0];
    if (py0 < sc[1]) py0 = sc[1];
    if (px1 > sc[0] + sc[2] - 1) px1 = sc[0] + sc[2] - 1;
    if (py1 > sc[1] + sc[3] - 1) py1 = sc[1] + sc[3] - 1;
    if (px0 > px1 || py0 > py1) return;
    /* depth plane */
    float fa = (float)area2;
    float e1x = (float)((int64_t)b.X - a.X), e1y = (float)((int64_t)b.Y - a.Y);
    float e2x = (float)((int64_t)c.X - a.X), e2y = (float)((int64_t)c.Y - a.Y);
    float d1 = b.D - a.D, d2 = c.D - a.D;
    float gx = (d1 * e2y - d2 * e1y) / fa;
    float gy = (d2 * e1x - d1 * e2x) / fa;
    float ox = (float)((int64_t)sc[0] * 256 + 128 - a.X), oy = (float)((int64_t)sc[1] * 256 + 128 - a.Y);
    float c0 = (a.D + gx * ox) + gy * oy;
    float ax = gx * 256.0f, ay = gy * 256.0f;
    sv v[3] = {a, b, c};
    int tl[3];
    for (int k = 0; k < 3; k++) {
        sv p = v[k], q = v[(k + 1) % 3];
        tl[k] = (q.Y < p.Y) || (q.Y == p.Y && q.X < p.X);
    }
    for (int64_t py = py0; py <= py1; py++) {
        int64_t PY = py * 256 + 128;
        for (int64_t px = px0; px <= px1; px++) {
            int64_t PX = px * 256 + 128;
            int inside = 1;
            for (int k = 0; k < 3 && inside; k++) {
                sv p = v[k], q = v[(k + 1) % 3];
                int64_t e = ((int64_t)q.X - p.X) * (PY - p.Y) - ((int64_t)q.Y - p.Y) * (PX - p.X);
                if (!(e > 0 || (e == 0 && tl[k]))) inside = 0;
            }
            if (!inside) continue;
            float u = (float)(px - sc[0]), w = (float)(py - sc[1]);
            float D = (c0 + ax * u) + ay * w;
            uint64_t key = ((uint64_t)depth_ordinal(D) << 32) | id;
            uint64_t* z = &zbuf[(size_t)py * TW + (size_t)px];
            if (key < *z) *z = key;
        }
    }
}

static void raster_face(uint32_t W, const float* verts, uint32_t n, uint32_t shooter, int face, uint64_t* zbuf) {
    int vp[4], sc[4];
    orc_face_rects(W, 0, face, vp, sc);
    const float* sq = verts + 12 * (size_t)shooter;
    float m[16], fr[9];
    orc_face_mvp(sq, face, m);
    orc_patch_frame(sq, fr);
    const uint32_t TW = 2 * W;
    const float hw = 0.5f * (float)vp[2], hh = 0.5f * (float)vp[3];
    const float vx = (float)vp[0], vy = (float)vp[1];
    for (uint32_t p = 0; p < n; p++) {
        const float* q = verts + 12 * (size_t)p;
        int behind = 1;
        for (int k = 0; k < 4 && behind; k++) {
            float d = ((q[3 * k] - fr[0]) * fr[3] + (q[3 * k + 1] - fr[1]) * fr[4]) + (q[3 * k + 2] - fr[2]) * fr[5];
            if (!(d < 0)) behind = 0;
        }
        if (behind) continue;
        v4 cv[4];
        for (int k = 0; k < 4; k++) {
            float x = q[3 * k], y = q[3 * k + 1], z = q[3 * k + 2];
            cv[k].x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12];
            cv[k].y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13];
            cv[k].z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14];
            cv[k].w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15];
        }
        static const int tri[2][3] = {{0, 1, 2}, {0, 2, 3}};
        for (int t = 0; t < 2; t++) {
            v4 poly[12];
            for (int k = 0; k < 3; k++) poly[k] = cv[tri[t][k]];
            int pn = clip_polygon(poly, 3);
            if (pn < 3) continue;
            sv s[12];
            int ok = 1;
            for (int k = 0; k < pn; k++) {
                if (!(poly[k].w > 0)) { ok = 0; break; }
                float xd = poly[k].x / poly[k].w, yd = poly[k].y / poly[k].w;
                float xw = (xd + 1.0f) * hw + vx, yw = (yd + 1.0f) * hh + vy;
                s[k].X = (int32_t)llrintf(xw * 256.0f);
                s[k].Y = (int32_t)llrintf(yw * 256.0f);
                s[k].D = 1.0f / poly[k].w;
            }
            if (!ok) continue;
            for (int j = 1; j + 1 < pn; j++) raster_triangle(s[0], s[j], s[j + 1], p, sc, TW, zbuf);
        }
    }
}

void orc_render_hemicube(uint32_t W, const float* verts, uint32_t n, uint32_t shooter, uint32_t* items) {
    size_t res = (size_t)(2 * W) * (size_t)(W * 3 / 2);
    uint64_t* z = (uint64_t*)malloc(sizeof(uint64_t) * res);
    for (size_t i = 0; i < res; i++) z[i] = ~0ull;
    for (int f = 0; f < 5; f++) raster_face(W, verts, n, shooter, f, z);
    for (size_t i = 0; i < res; i++) items[i] = (z[i] == ~0ull) ? 0u : (uint32_t)(z[i] & 0xFFFFFFFFu) + 1u;
    free(z);
}

/* ------------------------------------------------------------------------- */
/* ProcessHemicube: source/Kernel_ProcessHemicube.h:9-70                      */
/* ------------------------------------------------------------------------- */
uint32_t orc_process_hemicube(uint32_t W, uint32_t k, uint32_t workitems_x, const uint32_t* items,
                              const float* ff_table, uint32_t* rec_hemi, uint32_t* rec_id,
                              float* rec_energy, uint32_t cap) {
    const uint32_t TW = 2 * W, TH = (uint32_t)(W * 1.5);
    uint32_t wx = workitems_x < TW ? workitems_x : TW; /* Config::freeze, source/Config.cpp:44 */
    uint32_t span = TW / wx;                          /* source/Main.cpp:555 */
    uint32_t gy = TH * k;
    gy = (gy + 255) / 256 * 256; /* round-up of source/Main.cpp:593-596 */
    uint32_t write_index = 0;
    for (uint32_t y = 0; y < gy; y++) {
        if (y >= TH * k) break;
        const float* ff = ff_table + (size_t)TW * (y % TH);
        const uint32_t* row = items + (size_t)TW * y;
        for (uint32_t g = 0; g < wx; g++) {
            int x0 = (int)(g * span < TW - 1 ? g * span : TW - 1);
            int x1 = (int)((uint32_t)x0 + span < TW ? (uint32_t)x0 + span : TW);
            int space = 0;
            uint32_t wid = 0;
            while (x0 < x1) {
                uint32_t id = row[x0];
                float e = 0;
                while (x0 < x1) {
                    if (row[x0] == id) {
                        e += ff[x0];
                        ++x0;
                    } else
                        break;
                }
                if (id > 0) {
                    if (!space) {
                        wid = write_index;
                        write_index += 4;
                        space = 3;
                    } else {
                        ++wid;
                        --space;
                    }
                    if (wid < cap) {
                        rec_hemi[wid] = y / TH;
                        rec_id[wid] = id - 1;
                        rec_energy[wid] = e;
                    }
                }
            }
            for (; space > 0; --space) {
                ++wid;
                if (wid < cap) {
                    rec_hemi[wid] = 0;
                    rec_id[wid] = 0;
                    rec_energy[wid] = 0;
                }
            }
        }
    }
    return write_index;
}

void orc_ff_from_records(uint32_t k, uint32_t n, uint32_t nrec, const uint32_t* rec_hemi,
                         const uint32_t* rec_id, const float* rec_energy, float* F) {
    memset(F, 0, sizeof(float) * (size_t)k * n);
    for (uint32_t hi = 0; hi < k; hi++)
        for (uint32_t i = 0; i < nrec; i++) {
            if (rec_id[i] >= n) continue;
            if (rec_hemi[i] != hi) continue;
            F[(size_t)hi * n + rec_id[i]] += rec_energy[i];
        }
}

void orc_ff_exact(uint32_t W, uint32_t k, uint32_t n, const uint32_t* items, float* F) {
    const size_t res = (size_t)(2 * W) * (W * 3 / 2);
    float* table = (float*)malloc(sizeof(float) * res);
    orc_ff_table(W, table);
    uint64_t* acc = (uint64_t*)calloc((size_t)n, sizeof(uint64_t));
    for (uint32_t h = 0; h < k; h++) {
        memset(acc, 0, sizeof(uint64_t) * n);
        const uint32_t* it = items + res * h;
        for (size_t i = 0; i < res; i++)
            if (it[i] && it[i] <= n) acc[it[i] - 1] += (uint64_t)(table[i] * 0x1p61f);
        for (uint32_t i = 0; i < n; i++) F[(size_t)h * n + i] = (float)acc[i] * 0x1p-61f;
    }
    free(acc);
    free(table);
}

/* ------------------------------------------------------------------------- */
/* Shooter selection                                                          */
/* ------------------------------------------------------------------------- */
static float len2(const float* v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }

void orc_topk_ref(const float* rad, uint32_t n, uint32_t K, uint32_t* ids, uint8_t* valid) {
    uint32_t* tops = (uint32_t*)malloc(sizeof(uint32_t) * (K + 2));
    uint32_t s = 0;
    for (uint32_t pi = 0; pi < n; pi++) {
        float e = len2(rad + 3 * (size_t)pi);
        if (s == 0 || (e > 0 && len2(rad + 3 * (size_t)tops[s - 1]) <= e)) {
            tops[s++] = pi;
            /* std::list::sort is stable: insertion sort ascending by energy */
            for (uint32_t i = 1; i < s; i++) {
                uint32_t v = tops[i];
                float ev = len2(rad + 3 * (size_t)v);
                uint32_t j = i;
                while (j > 0 && ev < len2(rad + 3 * (size_t)tops[j - 1])) {
                    tops[j] = tops[j - 1];
                    j--;
                }
                tops[j] = v;
            }
            for (uint32_t i = 0; i < s / 2; i++) {
                uint32_t t = tops[i];
                tops[i] = tops[s - 1 - i];
                tops[s - 1 - i] = t;
            }
            if (s > K) s = K;
        }
    }
    for (uint32_t i = 0; i < K; i++) {
        ids[i] = i < s ? tops[i] : 0;
        valid[i] = i < s;
    }
    free(tops);
}

void orc_patch_areas(const float* verts, uint32_t n, float* area) {
    for (uint32_t p = 0; p < n; p++) {
        const float* q = verts + 12 * (size_t)p;
        float ax = q[0] - q[6], ay = q[1] - q[7], az = q[2] - q[8];
        float bx = q[3] - q[9], by = q[4] - q[10], bz = q[5] - q[11];
        float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        area[p] = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
    }
}

void orc_topk_phys(const float* rad, const float* area, uint32_t n, uint32_t K, uint32_t* ids,
                   uint8_t* valid) {
    uint32_t* top = (uint32_t*)malloc(sizeof(uint32_t) * (K + 1));
    float* key = (float*)malloc(sizeof(float) * (K + 1));
    uint32_t s = 0;
    for (uint32_t i = 0; i < n; i++) {
        const float* r = rad + 3 * (size_t)i;
        float k = ((r[0] + r[1]) + r[2]) * area[i];
        if (!(k > 0)) continue;
        if (s == K && !(k > key[s - 1])) continue;
        uint32_t j = s < K ? s : K - 1;
        while (j > 0 && key[j - 1] < k) {
            key[j] = key[j - 1];
            top[j] = top[j - 1];
            j--;
        }
        key[j] = k;
        top[j] = i;
        if (s < K) s++;
    }
    for (uint32_t i = 0; i < K; i++) {
        ids[i] = i < s ? top[i] : 0;
        valid[i] = i < s;
    }
    free(top);
    free(key);
}

/* ------------------------------------------------------------------------- */
/* The shoot loop: source/Main.cpp:1137-1309                                  */
/* ------------------------------------------------------------------------- */
static double unshot_power(const float* rad, const float* area, uint32_t n) {
    double s = 0;
    for (uint32_t i = 0; i < n; i++)
        s += (double)area[i] * ((double)rad[3 * i] + (double)rad[3 * i + 1] + (double)rad[3 * i + 2]);
    return s;
}

int orc_shoot(uint32_t mode, uint32_t ff_kind, uint32_t W, uint32_t K, uint32_t workitems_x,
              const float* verts, const float* color, const float* rho, uint32_t n, float* rad,
              float* illum, uint32_t n_shots, double tol, int threads, orc_stats* st) {
    if (W < 2 || (W & 1u) || W > 2048 || K == 0 || n == 0) return -1;
    const size_t res = (size_t)(2 * W) * (W * 3 / 2);
    uint32_t* items = (uint32_t*)malloc(sizeof(uint32_t) * res * K);
    float* F = (float*)malloc(sizeof(float) * (size_t)K * n);
    float* table = (float*)malloc(sizeof(float) * res);
    orc_ff_table(W, table);
    float* area = (float*)malloc(sizeof(float) * n);
    orc_patch_areas(verts, n, area);
    uint32_t ids[4096];
    uint8_t valid[4096];
    float saved[4096 * 3];
    if (K > 4096) return -1;
    uint32_t cap = (uint32_t)(res * K + 4 * 8);
    uint32_t *rh = 0, *ri = 0;
    float* re = 0;
    if (ff_kind == ORC_FF_RECORDS) {
        rh = (uint32_t*)malloc(sizeof(uint32_t) * cap);
        ri = (uint32_t*)malloc(sizeof(uint32_t) * cap);
        re = (float*)malloc(sizeof(float) * cap);
    }
    double p0 = unshot_power(rad, area, n);
    memset(st, 0, sizeof(*st));
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    for (uint32_t shot = 0; shot < n_shots; shot++) {
        if (mode == ORC_MODE_REF)
            orc_topk_ref(rad, n, K, ids, valid);
        else
            orc_topk_phys(rad, area, n, K, ids, valid);
        for (uint32_t h = 0; h < K; h++)
            if (valid[h]) memcpy(saved + 3 * h, rad + 3 * (size_t)ids[h], 3 * sizeof(float));
        memset(items, 0, sizeof(uint32_t) * res * K);
        int total = (int)(K * 5);
#pragma omp parallel
        {
            uint64_t* z = (uint64_t*)malloc(sizeof(uint64_t) * res);
#pragma omp for schedule(dynamic, 1)
            for (int t = 0; t < total; t++) {
                uint32_t h = (uint32_t)t / 5;
                int f = t % 5;
                if (!valid[h]) continue;
                int vp[4], sc[4];
                orc_face_rects(W, 0, f, vp, sc);
                for (int y = sc[1]; y < sc[1] + sc[3]; y++)
                    for (int x = sc[0]; x < sc[0] + sc[2]; x++) z[(size_t)y * 2 * W + x] = ~0ull;
                raster_face(W, verts, n, ids[h], f, z);
                uint32_t* it = items + res * h;
                for (int y = sc[1]; y < sc[1] + sc[3]; y++)
                    for (int x = sc[0]; x < sc[0] + sc[2]; x++) {
                        uint64_t kz = z[(size_t)y * 2 * W + x];
                        it[(size_t)y * 2 * W + x] = (kz == ~0ull) ? 0u : (uint32_t)(kz & 0xFFFFFFFFu) + 1u;
                    }
            }
            free(z);
        }
        for (uint32_t h = 0; h < K; h++) st->hemicubes += valid[h] ? 1.0 : 0.0;
        if (ff_kind == ORC_FF_RECORDS) {
            uint32_t nrec = orc_process_hemicube(W, K, workitems_x, items, table, rh, ri, re, cap);
            if (nrec > cap) nrec = cap;
            orc_ff_from_records(K, n, nrec, rh, ri, re, F);
        } else {
            orc_ff_exact(W, K, n, items, F);
        }
        for (uint32_t h = 0; h < K; h++) {
            if (!valid[h]) continue;
            const float* Fh = F + (size_t)h * n;
            const float* sv = saved + 3 * h;
            if (mode == ORC_MODE_REF) {
                const float* col = color + 3 * (size_t)ids[h];
                for (uint32_t i = 0; i < n; i++)
                    for (int c = 0; c < 3; c++) {
                        float t = sv[c] * Fh[i];
                        t = t * ORC_REFLECTIVITY;
                        t = t * col[c];
                        rad[3 * (size_t)i + c] = rad[3 * (size_t)i + c] + t;
                    }
            } else {
                float as = area[ids[h]];
                for (uint32_t i = 0; i < n; i++) {
                    if (!(area[i] > 0)) continue;
                    float g = (Fh[i] * as) / area[i];
                    for (int c = 0; c < 3; c++) {
                        float t = sv[c] * g;
                        t = rho[3 * (size_t)i + c] * t;
                        rad[3 * (size_t)i + c] = rad[3 * (size_t)i + c] + t;
                    }
                }
            }
        }
        float last[3] = {0, 0, 0};
        for (uint32_t h = 0; h < K; h++) {
            if (!valid[h]) continue;
            float* r = rad + 3 * (size_t)ids[h];
            float* il = illum + 3 * (size_t)ids[h];
            for (int c = 0; c < 3; c++) {
                last[c] = r[c];
                il[c] = il[c] + saved[3 * h + c];
                r[c] = r[c] - saved[3 * h + c];
            }
        }
        st->shots_done = shot + 1;
        memcpy(st->last_energy, last, sizeof(last));
        if (mode == ORC_MODE_REF) {
            if (sqrtf(last[0] * last[0] + last[1] * last[1] + last[2] * last[2]) < 0.1) {
                st->stopped = 1;
                break;
            }
        } else {
            st->residual = p0 > 0 ? unshot_power(rad, area, n) / p0 : 0.0;
            if (st->residual <= tol) {
                st->stopped = 1;
                break;
            }
        }
    }
    if (mode != ORC_MODE_REF && !st->stopped) st->residual = p0 > 0 ? unshot_power(rad, area, n) / p0 : 0.0;
    free(items);
    free(F);
    free(table);
    free(area);
    free(rh);
    free(ri);
    free(re);
    return 0;
}
