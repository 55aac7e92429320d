// C entry points over the reference's own CPU classes (compiled by build_ref.sh).
//
// TEST INFRASTRUCTURE ONLY.  Each function drives reference code exactly as the
// reference's shoot loop does and copies results into flat arrays so that the
// pytest suite (via ctypes) can pin the oracle restatement and the product's
// host-side code against it:
//   ref_scene_*      ModelContainer::load + updateData      (source/ModelContainer.cpp:35-56,81-155)
//   ref_ff_table     precomputeHemicubeFormFactors           (source/FormFactors.cpp:280-339)
//   ref_topk         ModelContainer::getHighestRadiosityPatchesId (source/ModelContainer.cpp:259-299)
//   ref_face_mvp     the per-face MVP of the shoot loop      (source/Main.cpp:1166-1184)
//   ref_config_*     Config::freeze and its getters          (source/Config.cpp:30-48)
//   ref_neighbours   Patch::neighbours as scene indices      (source/Patch.cpp:128-219)
//   ref_smooth_shade Colors::smoothShadePatch per patch      (source/Colors.cpp:198-262)
//   ref_highest_id   ModelContainer::getHighestRadiosityPatchId (source/ModelContainer.cpp:222-237)
//   ref_obj_*        WaveFrontModel + ModelContainer         (source/WaveFrontModel.cpp:15-143)
//   ref_rr_save      SaveToFile's Patch array and byte dump  (source/Main.cpp:1592-1625)
//   ref_rr_load      LoadFromFile + LoadingModel             (source/Main.cpp:1492-1517, source/LoadingModel.cpp:4-17)
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <list>
#include <sstream>
#include <string>
#include <vector>
#define private public   // lets the driver un-freeze the static Config between cases
#define protected public // reads Patch::vec1..vec4 for the flat vertex export
#include "Config.h"
#include "FormFactors.h"
#include "ModelContainer.h"
#include "Camera.h"
#include "Colors.h"
#include "LoadingModel.h"
#include "Transform.h"
#include "WaveFrontModel.h"
#undef private
#undef protected
#include <cstring>

static ModelContainer* g_scene = 0;
static ModelContainer* g_obj = 0;

// Scene index of every neighbour pointer of container m's patches (N x 8).
static void neighbours_of(ModelContainer* m, unsigned* nb) {
    unsigned n = m->getPatchesCount();
    Patch** p = m->getPatches();
    std::vector<std::pair<Patch*, unsigned> > idx(n);
    for (unsigned i = 0; i < n; i++) idx[i] = std::make_pair(p[i], i);
    std::sort(idx.begin(), idx.end());
    for (unsigned i = 0; i < n; i++)
        for (unsigned j = 0; j < 8; j++) {
            std::pair<Patch*, unsigned> key(p[i]->neighbours[j], 0);
            std::vector<std::pair<Patch*, unsigned> >::iterator it = std::lower_bound(idx.begin(), idx.end(), key);
            nb[8 * i + j] = (it != idx.end() && it->first == key.first) ? it->second : 0xFFFFFFFFu;
        }
}

static void export_of(ModelContainer* m, float* vertices, float* color, float* rad, float* illum) {
    unsigned n = m->getPatchesCount();
    if (vertices) std::memcpy(vertices, m->getVertices(), sizeof(float) * m->getVerticesCount());
    Patch** p = m->getPatches();
    for (unsigned i = 0; i < n; i++) {
        Vector3f c = p[i]->getColor();
        if (color) { color[3 * i] = c.x; color[3 * i + 1] = c.y; color[3 * i + 2] = c.z; }
        if (rad) { rad[3 * i] = p[i]->radiosity.x; rad[3 * i + 1] = p[i]->radiosity.y; rad[3 * i + 2] = p[i]->radiosity.z; }
        if (illum) {
            illum[3 * i] = p[i]->illumination.x; illum[3 * i + 1] = p[i]->illumination.y;
            illum[3 * i + 2] = p[i]->illumination.z;
        }
    }
}

static void config_set(unsigned W, unsigned K, unsigned wx) {
    Config::frozen = false;
    Config::setHemicubeSide(W);
    Config::setHemicubesCount(K);
    Config::setOCLWorkitemsX(wx);
    Config::freeze();
}

extern "C" {

// Builds the reference scene (ROOM + ROOMCLOSURE + CUBE + BLOCK) subdivided to
// `area` and returns its patch count.
unsigned ref_scene_build(double area) {
    delete g_scene;
    g_scene = new ModelContainer();
    g_scene->load();
    g_scene->maxPatchArea = area;
    return g_scene->getPatchesCount();
}

// Copies the scene: vertices N*12, indices N*6, color/radiosity/illumination N*3.
void ref_scene_get(float* vertices, int* indices, float* color, float* rad, float* illum) {
    unsigned n = g_scene->getPatchesCount();
    std::memcpy(vertices, g_scene->getVertices(), sizeof(float) * g_scene->getVerticesCount());
    std::memcpy(indices, g_scene->getIndices(), sizeof(int) * g_scene->getIndicesCount());
    Patch** p = g_scene->getPatches();
    for (unsigned i = 0; i < n; i++) {
        Vector3f c = p[i]->getColor();
        color[3 * i] = c.x; color[3 * i + 1] = c.y; color[3 * i + 2] = c.z;
        rad[3 * i] = p[i]->radiosity.x; rad[3 * i + 1] = p[i]->radiosity.y; rad[3 * i + 2] = p[i]->radiosity.z;
        illum[3 * i] = p[i]->illumination.x; illum[3 * i + 1] = p[i]->illumination.y;
        illum[3 * i + 2] = p[i]->illumination.z;
    }
}

// Derived Config values after freeze: out[0..8] = HEMICUBE_W, HEMICUBE_H, PATCHVIEW_TEX_W,
// PATCHVIEW_TEX_H, PATCHVIEW_TEX_RES, OCL_WORKITEMS_X, OCL_WORKITEMS_Y, HEMICUBES_CNT,
// span length (TEX_W / OCL_WORKITEMS_X as in source/Main.cpp:555).
void ref_config(unsigned W, unsigned K, unsigned wx, unsigned* out) {
    config_set(W, K, wx);
    out[0] = Config::HEMICUBE_W(); out[1] = Config::HEMICUBE_H();
    out[2] = Config::PATCHVIEW_TEX_W(); out[3] = Config::PATCHVIEW_TEX_H();
    out[4] = Config::PATCHVIEW_TEX_RES(); out[5] = Config::OCL_WORKITEMS_X();
    out[6] = Config::OCL_WORKITEMS_Y(); out[7] = Config::HEMICUBES_CNT();
    out[8] = Config::PATCHVIEW_TEX_W() / Config::OCL_WORKITEMS_X();
}

// K stacked copies of the texture-layout delta form-factor table (3*W*W*K floats).
void ref_ff_table(unsigned W, unsigned K, float* out) {
    config_set(W, K, 4);
    float* t = precomputeHemicubeFormFactors();
    std::memcpy(out, t, sizeof(float) * Config::PATCHVIEW_TEX_RES() * K);
    delete[] t;
}

// Sets every patch's radiosity (N*3) and runs the reference's top-K selection.
// ids[k] / valid[k] receive p_emitters_ids / (p_emitters != NULL).
void ref_topk(unsigned K, const float* rad, unsigned* ids, int* valid) {
    unsigned n = g_scene->getPatchesCount();
    Patch** p = g_scene->getPatches();
    for (unsigned i = 0; i < n; i++)
        p[i]->radiosity = Vector3f(rad[3 * i], rad[3 * i + 1], rad[3 * i + 2]);
    Patch** em = new Patch*[K];
    g_scene->getHighestRadiosityPatchesId(K, em, ids);
    for (unsigned k = 0; k < K; k++) valid[k] = em[k] != 0;
    delete[] em;
}

// MVP of hemicube face `i` (loop index: 0 UP, 1 DOWN, 2 LEFT, 3 RIGHT, 4 FRONT,
// source/Main.h:210-211) looking from the quad `q` (4 vertices, 12 floats).
// Column-major f[col][row] copied to out[col*4+row].
void ref_face_mvp(const float* q, int i, float* out) {
    static const Camera::PatchLook perm[5] = {Camera::PATCH_LOOK_UP, Camera::PATCH_LOOK_DOWN,
        Camera::PATCH_LOOK_LEFT, Camera::PATCH_LOOK_RIGHT, Camera::PATCH_LOOK_FRONT};
    Patch patch(Vector3f(q[0], q[1], q[2]), Vector3f(q[3], q[4], q[5]), Vector3f(q[6], q[7], q[8]),
                Vector3f(q[9], q[10], q[11]));
    Camera cam;
    Matrix4f proj;
    CGLTransform::Perspective(proj, 90, 1.0f, 0.01f, 1000);
    Matrix4f mv;
    mv.Identity();
    cam.lookFromPatch(&patch, perm[i]);
    mv *= cam.GetMatrix();
    Matrix4f mvp = proj * mv;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) out[c * 4 + r] = mvp[c][r];
}

// Patch getters of source/Patch.cpp:253-276 for the quad q: out = center(3), normal(3), up(3).
void ref_patch_frame(const float* q, float* out) {
    Patch patch(Vector3f(q[0], q[1], q[2]), Vector3f(q[3], q[4], q[5]), Vector3f(q[6], q[7], q[8]),
                Vector3f(q[9], q[10], q[11]));
    Vector3f c = patch.getCenter(), n = patch.getNormal(), u = patch.getUp();
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
    out[3] = n.x; out[4] = n.y; out[5] = n.z;
    out[6] = u.x; out[7] = u.y; out[8] = u.z;
}

// Display neighbours of the reference scene (after ref_scene_build), N x 8 scene indices.
void ref_neighbours(unsigned* nb) { neighbours_of(g_scene, nb); }

// Sets every patch's radiosity and illumination (N*3 each) and writes
// Colors::smoothShadePatch of every patch (N*12), as the display update does.
void ref_smooth_shade(const float* rad, const float* illum, float* colors) {
    unsigned n = g_scene->getPatchesCount();
    Patch** p = g_scene->getPatches();
    for (unsigned i = 0; i < n; i++) {
        p[i]->radiosity = Vector3f(rad[3 * i], rad[3 * i + 1], rad[3 * i + 2]);
        p[i]->illumination = Vector3f(illum[3 * i], illum[3 * i + 1], illum[3 * i + 2]);
    }
    for (unsigned i = 0; i < n; i++) Colors::smoothShadePatch(colors + 12 * i, p[i]);
}

// Sets every patch's radiosity and returns getHighestRadiosityPatchId.
unsigned ref_highest_id(const float* rad) {
    unsigned n = g_scene->getPatchesCount();
    Patch** p = g_scene->getPatches();
    for (unsigned i = 0; i < n; i++) p[i]->radiosity = Vector3f(rad[3 * i], rad[3 * i + 1], rad[3 * i + 2]);
    return g_scene->getHighestRadiosityPatchId();
}

// Loads an OBJ file through WaveFrontModel into a container subdivided to `area`;
// returns the patch count.
unsigned ref_obj_build(const char* path, double area) {
    delete g_obj;
    g_obj = new ModelContainer();
    g_obj->maxPatchArea = area;
    g_obj->addModel(new WaveFrontModel(path));
    return g_obj->getPatchesCount();
}

void ref_obj_get(float* vertices, float* color, float* rad, float* illum, unsigned* nb) {
    export_of(g_obj, vertices, color, rad, illum);
    if (nb) neighbours_of(g_obj, nb);
}

// SaveToFile's file contents for the reference scene with the given state: a 32-bit
// patch count (MSVC's unsigned long), then the Patch array with relative neighbours and
// NULL neighbour pointers, as raw bytes.  Returns the bytes written (out may be NULL to
// get the size); *record = sizeof(Patch) of this build.
unsigned long long ref_rr_save(const float* rad, const float* illum, unsigned char* out, unsigned* record) {
    unsigned n = g_scene->getPatchesCount();
    Patch** patches = g_scene->getPatches();
    *record = (unsigned)sizeof(Patch);
    unsigned long long bytes = 4 + (unsigned long long)n * sizeof(Patch);
    if (!out) return bytes;
    for (unsigned i = 0; i < n; i++) {
        patches[i]->radiosity = Vector3f(rad[3 * i], rad[3 * i + 1], rad[3 * i + 2]);
        patches[i]->illumination = Vector3f(illum[3 * i], illum[3 * i + 1], illum[3 * i + 2]);
    }
    Patch* data = new Patch[n];
    std::memset((void*)data, 0, sizeof(Patch) * n);  // padding bytes are otherwise indeterminate
    for (unsigned long i = 0; i < n; i++) data[i] = (*patches[i]);
    for (unsigned long i = 0; i < n; i++)
        for (unsigned int k = 0; k < 8; k++)
            for (unsigned long j = 0; j < n; j++)
                if (patches[i]->neighbours[k] == patches[j]) {
                    data[i].relativeNeighbours[k] = j;
                    data[i].neighbours[k] = NULL;
                    break;
                }
    const unsigned count = n;
    std::memcpy(out, &count, 4);
    std::memcpy(out + 4, (const void*)data, sizeof(Patch) * n);
    delete[] data;
    return bytes;
}

// LoadFromFile on file bytes of this build's Patch layout: a LoadingModel in a new
// container (no subdivision).  Returns the patch count; ref_obj_get reads the result.
unsigned ref_rr_load(const unsigned char* bytes) {
    unsigned count;
    std::memcpy(&count, bytes, 4);
    Patch* data = new Patch[count];
    std::memcpy((void*)data, bytes + 4, sizeof(Patch) * count);
    delete g_obj;
    g_obj = new ModelContainer();
    g_obj->maxPatchArea = 0;
    g_obj->addModel(new LoadingModel(data, count));
    delete[] data;
    return g_obj->getPatchesCount();
}

}  // extern "C"
