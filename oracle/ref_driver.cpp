// C entry points over the reference's own CPU classes (compiled by build_ref.sh).
//
// TEST INFRASTRUCTURE ONLY.  Each function drives reference code exactly as the
// reference's shoot loop does and copies results into flat arrays so that the
// pytest suite (via ctypes) can pin the oracle restatement and the product's
// host-side code against it:
//   ref_scene_*      ModelContainer::load + updateData      (source/ModelContainer.cpp:89-209)
//   ref_ff_table     precomputeHemicubeFormFactors           (source/FormFactors.cpp:280-339)
//   ref_topk         ModelContainer::getHighestRadiosityPatchesId (source/ModelContainer.cpp:313-353)
//   ref_face_mvp     the per-face MVP of the shoot loop      (source/Main.cpp:1166-1184)
//   ref_config_*     Config::freeze and its getters          (source/Config.cpp:30-48)
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
#include "Transform.h"
#undef private
#undef protected
#include <cstring>

static ModelContainer* g_scene = 0;

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

}  // extern "C"
