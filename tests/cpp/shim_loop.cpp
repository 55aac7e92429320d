// Reference-style driver of the C++ shim: the OnIdle shoot section of
// source/Main.cpp:1124-1309 expressed with Config / ModelContainer / Patch.
// Usage: shim_loop <hemicube> <hemicubes> <area> <max_shots> <out.bin>
// Writes N (uint32), shots (uint32), then radiosity and illumination (N*3 floats each).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "radiosity_shim.hpp"

using rad::Config;

int main(int argc, char** argv) {
    if (argc != 6) return 2;
    Config::setHemicubeSide((unsigned)std::atoi(argv[1]));
    Config::setHemicubesCount((unsigned)std::atoi(argv[2]));
    Config::setMaxPatchArea(std::atof(argv[3]));
    Config::setShootsPerCycle((unsigned)std::atoi(argv[4]));
    Config::freeze();
    Config::setHemicubeSide(999);  // ignored after freeze, as in the reference
    rad::ModelContainer scene;
    scene.load();
    scene.maxPatchArea = Config::MAX_PATCH_AREA();
    std::vector<rad::Patch*> em(Config::HEMICUBES_CNT());
    std::vector<unsigned> ids(Config::HEMICUBES_CNT());
    scene.getHighestRadiosityPatchesId(Config::HEMICUBES_CNT(), em.data(), ids.data());
    rad_stats st;
    scene.shoot(Config::SHOOTS_PER_CYCLE(), &st);
    unsigned n = scene.getPatchesCount();
    FILE* f = std::fopen(argv[5], "wb");
    if (!f) return 3;
    unsigned shots = st.shots_done;
    std::fwrite(&n, 4, 1, f);
    std::fwrite(&shots, 4, 1, f);
    rad::Patch** p = scene.getPatches();
    for (unsigned i = 0; i < n; i++) std::fwrite(&p[i]->radiosity, 4, 3, f);
    for (unsigned i = 0; i < n; i++) std::fwrite(&p[i]->illumination, 4, 3, f);
    std::fclose(f);
    std::printf("patches %u shots %u stopped %u first emitter %u (%s) W %u\n", n, shots, st.stopped, ids[0],
                em[0] ? "valid" : "null", Config::HEMICUBE_W());
    return 0;
}
