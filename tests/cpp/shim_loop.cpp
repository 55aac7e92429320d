// Reference-style driver of the C++ shim: the OnIdle shoot section of
// source/Main.cpp:1124-1309 expressed with Config / ModelContainer / Patch.
// Usage: shim_loop <hemicube> <hemicubes> <area> <max_shots> <out.bin>
// Writes N (uint32), shots (uint32), radiosity and illumination (N*3 floats each), the
// highest-radiosity patch id, a flag (1 = the state saved to <out.bin>.rr and loaded back
// equals the solved one) and the display colours (N*12 floats).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
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
    // the display update, the single-patch selection and a save / load round trip
    const unsigned hid = scene.getHighestRadiosityPatchId();
    std::vector<float> colors, radiative;
    scene.updateDisplayColors(colors, radiative);
    std::string rr = std::string(argv[5]) + ".rr";
    scene.saveToFile(rr.c_str());
    rad::ModelContainer back;
    back.loadFromFile(rr.c_str());
    unsigned same = back.getPatchesCount() == n && back.getHighestRadiosityPatchId() == hid;
    rad::Patch** p = scene.getPatches();
    rad::Patch** q = back.getPatches();
    std::map<rad::Patch*, unsigned> index;  // patches are separate objects: map pointers to indices
    for (unsigned i = 0; i < n; i++) index[p[i]] = i;
    for (unsigned i = 0; same && i < n; i++) {
        same = std::memcmp(&p[i]->radiosity, &q[i]->radiosity, 12) == 0 &&
               std::memcmp(&p[i]->illumination, &q[i]->illumination, 12) == 0;
        for (int j = 0; same && j < 8; j++) same = q[i]->getNeighbours()[j] == q[index[p[i]->getNeighbours()[j]]];
    }
    FILE* f = std::fopen(argv[5], "wb");
    if (!f) return 3;
    unsigned shots = st.shots_done;
    std::fwrite(&n, 4, 1, f);
    std::fwrite(&shots, 4, 1, f);
    for (unsigned i = 0; i < n; i++) std::fwrite(&p[i]->radiosity, 4, 3, f);
    for (unsigned i = 0; i < n; i++) std::fwrite(&p[i]->illumination, 4, 3, f);
    std::fwrite(&hid, 4, 1, f);
    std::fwrite(&same, 4, 1, f);
    std::fwrite(colors.data(), 4, colors.size(), f);
    std::fclose(f);
    std::printf("patches %u shots %u stopped %u first emitter %u (%s) W %u highest %u reload %u\n", n, shots,
                st.stopped, ids[0], em[0] ? "valid" : "null", Config::HEMICUBE_W(), hid, same);
    return 0;
}
