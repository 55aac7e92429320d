/* oracle.h - CPU restatement of the reference's progressive-refinement hemicube
 * shoot loop (david-sabata/Radiosity).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm load this library, and only as the checker or the
 * timed CPU baseline.  The product (radiosity_gb300) never links or calls it.
 *
 * Pinning: the delta form-factor table, the face cameras / MVPs, the scene
 * geometry and the top-K shooter selection are pinned bit-for-bit against the
 * reference's own C++ compiled by oracle/build_ref.sh (tests/test_oracle_pins.py,
 * golden fixtures in tests/golden/).  The reference's hemicube render is OpenGL
 * fixed-function rasterisation, which cannot run on these machines (no graphics
 * stack): the raster rules restated here (orc_render_hemicube) are this
 * project's contract, written to follow GL's documented behaviour; that part is
 * parity-unpinned against the reference itself.
 */
#ifndef RADIOSITY_ORACLE_H
#define RADIOSITY_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Face loop index, source/Main.cpp:1164 with p_patchlook_perm of source/Main.h:210. */
enum { ORC_FACE_UP = 0, ORC_FACE_DOWN = 1, ORC_FACE_LEFT = 2, ORC_FACE_RIGHT = 3, ORC_FACE_FRONT = 4 };

/* Delta form-factor table in texture layout, one hemicube: 2W x 1.5W floats,
 * row-major with row 0 at the bottom.  Restates Calc_HemicubeFormFactors
 * (source/FormFactors.cpp:23-67) and the layout copy of
 * precomputeHemicubeFormFactors (source/FormFactors.cpp:295-314). */
int orc_ff_table(uint32_t W, float* out);

/* The reference's delta-FF self-check sum: 4*sum(side) + sum(front) in float, in
 * the loop order of source/FormFactors.cpp:89-104. */
float orc_ff_sum(uint32_t W);

/* Viewport and scissor rectangles (x, y, w, h) of face i of hemicube hi,
 * source/Main.cpp:316-389.  Row offset of hemicube hi is int(1.5*W*hi). */
void orc_face_rects(uint32_t W, uint32_t hi, int face, int vp[4], int sc[4]);

/* Column-major MVP (out[col*4+row]) of face `face` looking from quad q (12
 * floats), restating Camera::lookFromPatch, CGLTransform::LookAt/Perspective/
 * Frustum and Matrix4f products (source/Camera.cpp:19-52,97-103,
 * source/Transform.cpp:26-80,127-156, source/Vector.cpp:445-527,
 * source/Main.cpp:1170-1183). */
void orc_face_mvp(const float* q, int face, float* out);

/* Center / normal / up of a quad (source/Patch.cpp:253-276). */
void orc_patch_frame(const float* q, float* out9);

/* Item buffer of one hemicube: 2W x 1.5W uint32, 0 = nothing, else patch+1.
 * Local (hemicube-relative) window coordinates are used, so the result does not
 * depend on the hemicube's slot in a batch.  Rules (the raster contract):
 *  - quad p = triangles (v0,v1,v2),(v0,v2,v3) (source/ModelContainer.cpp:112-117)
 *  - patches with all 4 vertices strictly behind the shooter plane are skipped
 *  - clip space c_r = ((m0r*x + m1r*y) + m2r*z) + m3r
 *  - Sutherland-Hodgman clip against z+w>=0, w-z>=0, 1024w-x>=0, 1024w+x>=0,
 *    1024w-y>=0, 1024w+y>=0 (in that order), fan re-triangulation
 *  - window x = ((x/w + 1) * (0.5*vp_w)) + vp_x, snapped to 1/256 px (rint)
 *  - CCW front, area<=0 culled, pixel centres at +0.5, top-left fill rule
 *  - depth = 1/w, plane-interpolated in float; key (depth_ordinal<<32 | patch)
 *    with min-key wins, i.e. GL_LESS with patch-index draw order.
 * Pixels outside the face's scissor are never written. */
void orc_render_hemicube(uint32_t W, const float* verts, uint32_t n, uint32_t shooter, uint32_t* items);

/* Restatement of the ProcessHemicube OpenCL kernel (source/Kernel_ProcessHemicube.h:9-70)
 * over k stacked item buffers, executed work-item by work-item in the order
 * (y, x-span).  Returns the final write index (records incl. zero padding);
 * records past `cap` are counted but not stored. */
uint32_t orc_process_hemicube(uint32_t W, uint32_t k, uint32_t workitems_x, const uint32_t* items,
                              const float* ff_table, uint32_t* rec_hemi, uint32_t* rec_id,
                              float* rec_energy, uint32_t cap);

/* Host accumulation of records into per-hemicube form-factor rows F[k][n]
 * (source/Main.cpp:1251-1269) in record order, float. */
void orc_ff_from_records(uint32_t k, uint32_t n, uint32_t nrec, const uint32_t* rec_hemi,
                         const uint32_t* rec_id, const float* rec_energy, float* F);

/* Form-factor rows as exact sums: every pixel's delta FF is an integer multiple
 * of 2^-61 for W <= 2048, so the sum is carried exactly in uint64 and rounded
 * once to float.  This is the product's arithmetic contract. */
void orc_ff_exact(uint32_t W, uint32_t k, uint32_t n, const uint32_t* items, float* F);

/* Top-K selection of ModelContainer::getHighestRadiosityPatchesId
 * (source/ModelContainer.cpp:259-299), simulated literally (list append, stable
 * ascending sort, reverse, truncate).  rad is n*3; ids[k], valid[k]. */
void orc_topk_ref(const float* rad, uint32_t n, uint32_t K, uint32_t* ids, uint8_t* valid);

/* PHYS selection: top-K by unshot power (r+g+b)*area, ties to lower index,
 * zero power never selected. */
void orc_topk_phys(const float* rad, const float* area, uint32_t n, uint32_t K, uint32_t* ids,
                   uint8_t* valid);

/* Quad area used by PHYS mode: 0.5*|d1 x d2| of the diagonals, float. */
void orc_patch_areas(const float* verts, uint32_t n, float* area);

enum { ORC_MODE_REF = 0, ORC_MODE_PHYS = 1 };
enum { ORC_FF_EXACT = 0, ORC_FF_RECORDS = 1 };

typedef struct {
    uint32_t shots_done;     /* batches executed */
    uint32_t stopped;        /* stop rule fired */
    float last_energy[3];    /* REF: lastEnergy of source/Main.cpp:1287-1298 */
    double residual;         /* PHYS: unshot power / initial power (FP64 sum) */
    double hemicubes;        /* hemicubes rendered */
} orc_stats;

/* Runs up to n_shots batches of the shoot loop (source/Main.cpp:1137-1309) on the
 * state arrays in place (rad = unshot "radiosity", illum = "illumination",
 * both n*3).  REF mode: receiver += ((saved*F)*0.3)*shooter_color.  PHYS mode:
 * receiver += rho_j*saved*(F*A_i/A_j), stop when residual <= tol.
 * ff_kind selects exact sums (product contract) or the record path.
 * threads: OpenMP threads for the per-face raster (0 = default). */
int orc_shoot(uint32_t mode, uint32_t ff_kind, uint32_t W, uint32_t K, uint32_t workitems_x,
              const float* verts, const float* color, const float* rho, uint32_t n, float* rad,
              float* illum, uint32_t n_shots, double tol, int threads, orc_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
