// radiosity_shim.hpp - header-only C++ adapter that keeps the reference's
// Config / FormFactors / ModelContainer / Patch call sites
// (source/Config.h:6-37, source/FormFactors.h:20, source/ModelContainer.h:11-53,
// source/Patch.h:16-56) compiling on top of the C ABI in radiosity.h.
//
// The reference's OnIdle shoot section (source/Main.cpp:1124-1309) becomes
//     rad::ModelContainer scene; scene.load(); scene.maxPatchArea = Config::MAX_PATCH_AREA();
//     scene.shoot(Config::SHOOTS_PER_CYCLE());           // GPU: select, render, reduce, update
//     Patch** p = scene.getPatches();                    // radiosity / illumination synced back
// Differences from the reference: Patch objects are host copies refreshed by shoot();
// writing Patch::radiosity and calling scene.pushState() uploads edits.  The display
// update of source/Main.cpp:1318-1372 is scene.updateDisplayColors(colors, radiative)
// (all patches at once on the GPU, Colors::smoothShadePatch per patch); SaveToFile /
// LoadFromFile (source/Main.cpp:1460-1647) are scene.saveToFile(path) /
// scene.loadFromFile(path) without the file dialogs; scene.loadObj(path) adds a
// WaveFrontModel (source/WaveFrontModel.cpp:15-143) instead of the built-in scene.
#pragma once
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

#include "radiosity.h"

namespace rad {

struct Vector3f {
    float x = 0, y = 0, z = 0;
    Vector3f() = default;
    Vector3f(float a, float b, float c) : x(a), y(b), z(c) {}
};

// Static, freezable configuration with the reference's setters and getters.
class Config {
  public:
    static void setHemicubeSide(unsigned n) { set(cfg().hemicube_side, n); }
    static void setOCLWorkitemsX(unsigned n) { set(cfg().ocl_workitems_x, n); }
    static void setMaxPatchArea(double n) {
        if (frozen()) return warn();
        cfg().max_patch_area = n;
    }
    static void setShootsPerCycle(unsigned n) { set(cfg().shoots_per_cycle, n); }
    static void setHemicubesCount(unsigned n) { set(cfg().hemicubes_count, n); }
    static void freeze() {
        frozen() = true;
        rad_config_derived(&cfg(), derived());
    }
    static unsigned HEMICUBE_W() { return derived()[0]; }
    static unsigned HEMICUBE_H() { return derived()[1]; }
    static unsigned PATCHVIEW_TEX_W() { return derived()[2]; }
    static unsigned PATCHVIEW_TEX_H() { return derived()[3]; }
    static unsigned PATCHVIEW_TEX_RES() { return derived()[4]; }
    static double MAX_PATCH_AREA() { return cfg().max_patch_area; }
    static unsigned OCL_WORKITEMS_X() { return derived()[5]; }
    static unsigned OCL_WORKITEMS_Y() { return derived()[6]; }
    static unsigned SHOOTS_PER_CYCLE() { return cfg().shoots_per_cycle; }
    static unsigned HEMICUBES_CNT() { return cfg().hemicubes_count; }
    static rad_config& cfg() {
        static rad_config c = [] {
            rad_config d;
            rad_config_default(&d);
            return d;
        }();
        return c;
    }

  private:
    static bool& frozen() {
        static bool f = false;
        return f;
    }
    static uint32_t* derived() {
        static uint32_t d[9] = {0};
        return d;
    }
    static void warn() { std::fprintf(stderr, "Error: Trying to modify frozen configuration\n"); }
    static void set(uint32_t& field, unsigned n) {
        if (frozen()) return warn();
        field = n;
    }
};

// The texture-layout delta form-factor table, HEMICUBES_CNT stacked copies; caller delete[]s it.
inline float* precomputeHemicubeFormFactors() {
    rad_ctx* ctx = nullptr;
    if (rad_create(&Config::cfg(), &ctx) != RAD_OK) throw std::runtime_error("rad_create failed");
    const unsigned copies = Config::HEMICUBES_CNT();
    float* out = new float[(size_t)Config::PATCHVIEW_TEX_RES() * copies];
    int rc = rad_ff_table(ctx, out, copies);
    rad_destroy(ctx);
    if (rc != RAD_OK) {
        delete[] out;
        throw std::runtime_error("rad_ff_table failed");
    }
    return out;
}

class Patch {
  public:
    Vector3f radiosity, illumination;
    Patch* neighbours[8] = {};  // display neighbours, numbered from the upper left corner (source/Patch.h:50)
    Vector3f getColor() const { return color; }
    float getReflectivity() const { return 0.3f; }  // REFLECTIVITY, source/Patch.h:13
    Patch** getNeighbours() { return neighbours; }
    Vector3f color;
};

class ModelContainer {
  public:
    double maxPatchArea = 0;
    ~ModelContainer() {
        if (ctx) rad_destroy(ctx);
        for (Patch* p : patches) delete p;
    }
    // ROOM + ROOMCLOSURE + CUBE + BLOCK of source/ModelContainer.cpp:35-56 (built lazily).
    void load() { loaded = true; }
    float* getVertices() { return refresh(), vertices.data(); }
    unsigned getVerticesCount() { return refresh(), (unsigned)vertices.size(); }
    int* getIndices() { return refresh(), indices.data(); }
    unsigned getIndicesCount() { return refresh(), (unsigned)indices.size(); }
    Patch** getPatches() { return refresh(), patches.data(); }
    unsigned getPatchesCount() { return refresh(), (unsigned)patches.size(); }
    // GPU top-K on the current state; NULL emitters get id 0 as in the reference.
    void getHighestRadiosityPatchesId(unsigned count, Patch** p_emitters, unsigned* p_emitters_ids) {
        device();
        std::vector<uint8_t> valid(Config::HEMICUBES_CNT());
        std::vector<uint32_t> ids(Config::HEMICUBES_CNT());
        check(rad_select_shooters(ctx, ids.data(), valid.data()));
        for (unsigned i = 0; i < count; i++) {
            bool v = i < ids.size() && valid[i];
            p_emitters_ids[i] = v ? ids[i] : 0;
            p_emitters[i] = v ? patches[ids[i]] : nullptr;
        }
    }
    // getHighestRadiosityPatchId (source/ModelContainer.cpp:222-237) on the device state.
    unsigned getHighestRadiosityPatchId() {
        device();
        uint32_t id = 0;
        check(rad_highest_patch(ctx, &id));
        return id;
    }
    // The display update after a batch of shots: colors = smoothShadePatch of every patch,
    // radiative = radiosity at the 4 corners (N*12 floats each, the VBO layout).
    void updateDisplayColors(std::vector<float>& colors, std::vector<float>& radiative) {
        device();
        colors.resize(12 * patches.size());
        radiative.resize(12 * patches.size());
        check(rad_display_colors(ctx, colors.data(), radiative.data()));
    }
    // SaveToFile without the dialog: the .rr file of this build's pointer width.
    void saveToFile(const char* path) {
        refresh();
        std::vector<float> r(3 * patches.size()), il(3 * patches.size());
        for (size_t i = 0; i < patches.size(); i++) {
            r[3 * i] = patches[i]->radiosity.x; r[3 * i + 1] = patches[i]->radiosity.y; r[3 * i + 2] = patches[i]->radiosity.z;
            il[3 * i] = patches[i]->illumination.x; il[3 * i + 1] = patches[i]->illumination.y;
            il[3 * i + 2] = patches[i]->illumination.z;
        }
        uint64_t bytes = 0;
        const uint32_t ptr = (uint32_t)sizeof(void*);
        check(rad_rr_size((uint32_t)patches.size(), ptr, &bytes));
        std::vector<unsigned char> buf((size_t)bytes);
        check(rad_rr_write((uint32_t)patches.size(), vertices.data(), color.data(), r.data(), il.data(),
                           neighbours.data(), ptr, buf.data(), bytes));
        std::ofstream f(path, std::ios::binary);
        f.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
        if (!f) throw std::runtime_error("radiosity: unable to write the file");
    }
    // LoadFromFile without the dialog: replaces the scene by the file's patches.
    void loadFromFile(const char* path) {
        std::ifstream f(path, std::ios::binary);
        std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        uint32_t n = 0, ptr = 0;
        check(rad_rr_read(buf.data(), buf.size(), 0, &n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &ptr));
        resize(n);
        check(rad_rr_read(buf.data(), buf.size(), n, &n, vertices.data(), indices.data(), color.data(),
                          radiosity0.data(), illumination0.data(), neighbours.data(), &ptr));
        rebuild();
    }
    // A WaveFrontModel subdivided to maxPatchArea in place of the built-in scene.
    void loadObj(const char* path) {
        std::ifstream f(path, std::ios::binary);
        std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        uint32_t n = 0;
        check(rad_scene_obj(text.data(), text.size(), maxPatchArea, 0, &n, nullptr, nullptr, nullptr, nullptr, nullptr,
                            nullptr));
        resize(n);
        check(rad_scene_obj(text.data(), text.size(), maxPatchArea, n, &n, vertices.data(), indices.data(),
                            color.data(), radiosity0.data(), illumination0.data(), neighbours.data()));
        rebuild();
    }
    // `shots` iterations of the shoot loop; returns true when the stop rule fired.
    bool shoot(unsigned shots, rad_stats* stats = nullptr) {
        device();
        rad_stats st;
        check(rad_shoot(ctx, shots, &st));
        pullState();
        if (stats) *stats = st;
        return st.stopped != 0;
    }
    void pushState() {
        device();
        std::vector<float> r(3 * patches.size()), il(3 * patches.size());
        for (size_t i = 0; i < patches.size(); i++) {
            r[3 * i] = patches[i]->radiosity.x; r[3 * i + 1] = patches[i]->radiosity.y; r[3 * i + 2] = patches[i]->radiosity.z;
            il[3 * i] = patches[i]->illumination.x; il[3 * i + 1] = patches[i]->illumination.y;
            il[3 * i + 2] = patches[i]->illumination.z;
        }
        check(rad_set_state(ctx, r.data(), il.data()));
    }
    void pullState() {
        std::vector<float> r(3 * patches.size()), il(3 * patches.size());
        check(rad_download(ctx, r.data(), il.data()));
        for (size_t i = 0; i < patches.size(); i++) {
            patches[i]->radiosity = Vector3f(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
            patches[i]->illumination = Vector3f(il[3 * i], il[3 * i + 1], il[3 * i + 2]);
        }
    }

  private:
    bool loaded = false, built = false;
    rad_ctx* ctx = nullptr;
    std::vector<float> vertices, color, radiosity0, illumination0;
    std::vector<int> indices;
    std::vector<uint32_t> neighbours;
    std::vector<Patch*> patches;

    void check(int rc) {
        if (rc != RAD_OK) throw std::runtime_error(std::string("radiosity: ") + rad_last_error(ctx));
    }
    void resize(uint32_t n) {
        vertices.resize(12 * (size_t)n);
        indices.resize(6 * (size_t)n);
        color.resize(3 * (size_t)n);
        radiosity0.resize(3 * (size_t)n);
        illumination0.resize(3 * (size_t)n);
        neighbours.resize(8 * (size_t)n);
    }
    // Patch objects from the flat arrays (a new scene: any device context is dropped).
    void rebuild() {
        if (ctx) rad_destroy(ctx);
        ctx = nullptr;
        for (Patch* p : patches) delete p;
        patches.clear();
        const size_t n = color.size() / 3;
        for (size_t i = 0; i < n; i++) {
            Patch* p = new Patch();
            p->color = Vector3f(color[3 * i], color[3 * i + 1], color[3 * i + 2]);
            p->radiosity = Vector3f(radiosity0[3 * i], radiosity0[3 * i + 1], radiosity0[3 * i + 2]);
            p->illumination = Vector3f(illumination0[3 * i], illumination0[3 * i + 1], illumination0[3 * i + 2]);
            patches.push_back(p);
        }
        for (size_t i = 0; i < n; i++)
            for (int j = 0; j < 8; j++) patches[i]->neighbours[j] = patches[neighbours[8 * i + j]];
        loaded = built = true;
    }
    void refresh() {
        if (!loaded || built) return;
        uint32_t n = 0;
        rad_scene_reference(maxPatchArea, 0, &n, nullptr, nullptr, nullptr, nullptr, nullptr);
        resize(n);
        rad_scene_reference(maxPatchArea, n, &n, vertices.data(), indices.data(), color.data(), radiosity0.data(),
                            illumination0.data());
        rad_scene_reference_neighbours(maxPatchArea, n, &n, neighbours.data());
        rebuild();
    }
    void device() {
        refresh();
        if (ctx) return;
        if (rad_create(&Config::cfg(), &ctx) != RAD_OK) throw std::runtime_error("rad_create failed");
        check(rad_upload_scene(ctx, vertices.data(), indices.data(), color.data(), nullptr, radiosity0.data(),
                               illumination0.data(), (uint32_t)patches.size()));
        check(rad_upload_neighbours(ctx, neighbours.data()));
    }
};

}  // namespace rad
