/* radiosity.h - C ABI of the GB300 progressive-refinement hemicube radiosity solver.
 *
 * Drop-in boundary for the reference's shoot loop (david-sabata/Radiosity,
 * source/Main.cpp:1124-1309).  The reference has no FFI; its "API" is the set of
 * C++ classes the loop calls.  Each entry point below names the reference code it
 * replaces.  All calls return an int status (RAD_OK = 0, negative = error) and
 * never throw or abort.  Host arrays are caller-owned and copied; device memory is
 * owned by the rad_ctx.  A rad_ctx is not thread-safe: one context per host thread.
 */
#ifndef RADIOSITY_GB300_H
#define RADIOSITY_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAD_OK 0
#define RAD_E_INVALID (-1)  /* bad argument (reference: cerr + ignore, source/Config.cpp:54-112) */
#define RAD_E_CUDA (-2)     /* CUDA runtime error (reference: _ASSERT on CL calls) */
#define RAD_E_OVERFLOW (-3) /* raster record or bin capacity exceeded; results of the call invalid */
#define RAD_E_STATE (-4)    /* call out of order (e.g. no scene uploaded) */
#define RAD_E_NOMEM (-5)    /* device allocation failed */
#define RAD_E_TIMEOUT (-6)  /* a bounded device wait gave up */
#define RAD_E_NOALLOC_LIMIT (-7) /* request larger than the allocation-free entry point's fixed scratch */
#define RAD_E_NUMERIC (-8)  /* an iterative solve met a non-finite residual (NaN / inf in its data) */

typedef enum { RAD_MODE_REF = 0, RAD_MODE_PHYS = 1 } rad_mode;

/* Mirrors the static Config of source/Config.h:6-37 plus the solver's own knobs. */
typedef struct rad_config {
    uint32_t hemicube_side;   /* Config::setHemicubeSide (default 16); even, 2..2048 */
    uint32_t ocl_workitems_x; /* Config::setOCLWorkitemsX (default 4); derived sizes only */
    uint32_t shoots_per_cycle;/* Config::setShootsPerCycle (default 500) */
    uint32_t hemicubes_count; /* Config::setHemicubesCount (default 10): shooters per batch K, 1..1024 */
    double max_patch_area;    /* Config::setMaxPatchArea (default 0.5) */
    uint32_t mode;            /* rad_mode: REF = the reference's update rule, PHYS = rho*F*Ai/Aj */
    uint32_t tile;            /* raster bin side in pixels: 16, 32 or 64; 0 = choose by W */
    double tolerance;         /* PHYS stop rule: unshot power / initial power <= tolerance */
    uint32_t tri_capacity;    /* raster records per hemicube (one per patch quad and face, up to 4 per
                                 clipped quad); 0 = 3*N + 4096 */
    uint32_t binref_capacity; /* bin references per hemicube; 0 = 4 * tri_capacity */
    int32_t device;           /* CUDA device ordinal */
    uint32_t small_tri_pixels;/* records whose box clamped to a bin is at most this many pixels (and whose
                                 extent is at most 64 px) are rasterised by exact row spans, the others
                                 by one warp per triangle; 1..4096, 0 = 4096 */
} rad_config;

typedef struct rad_stats {
    uint32_t shots_done;   /* batches (reference "shoot" iterations) executed by the call */
    uint32_t stopped;      /* 1 when the stop rule fired (source/Main.cpp:1298-1300) */
    float last_energy[3];  /* REF: lastEnergy of source/Main.cpp:1287-1295 */
    double residual;       /* PHYS: unshot power / initial power, FP64 sum */
    double hemicubes;      /* hemicubes rendered by the call */
    double device_ms;      /* device time of the call, CUDA events on the context stream */
} rad_stats;

typedef struct rad_ctx rad_ctx;

/* Defaults of source/Config.cpp:6-10 (hemicube 16, work-items 4, 500 shots,
 * area 0.5, 10 hemicubes), REF mode. */
int rad_config_default(rad_config* cfg);

/* Config::freeze derived values (source/Config.cpp:30-48): out[0..8] = HEMICUBE_W,
 * HEMICUBE_H, PATCHVIEW_TEX_W, PATCHVIEW_TEX_H, PATCHVIEW_TEX_RES, OCL_WORKITEMS_X,
 * OCL_WORKITEMS_Y, HEMICUBES_CNT, span length (source/Main.cpp:555). */
int rad_config_derived(const rad_config* cfg, uint32_t out[9]);

/* Creates a context on cfg->device: replaces InitGLObjects/InitCLObjects
 * (source/Main.cpp:11-611).  *out is NULL on failure. */
int rad_create(const rad_config* cfg, rad_ctx** out);

/* Releases every device resource (CleanupGLObjects/CleanupCLObjects, source/Main.cpp:616-670). */
int rad_destroy(rad_ctx* ctx);

/* Uploads the scene of ModelContainer::getVertices/getIndices/getPatches
 * (source/ModelContainer.cpp:161-219): vertices N*12 floats (4 corners per patch),
 * indices N*6 (may be NULL; if given it must be the (0,1,2,0,2,3)+4i pattern),
 * color N*3 (Patch::getColor), reflectance N*3 (PHYS only, may be NULL in REF),
 * radiosity N*3 (Patch::radiosity = unshot energy), illumination N*3. */
int rad_upload_scene(rad_ctx* ctx, const float* vertices, const int32_t* indices, const float* color,
                     const float* reflectance, const float* radiosity, const float* illumination,
                     uint32_t n);

/* Replaces the radiosity / illumination state (either may be NULL to keep it). */
int rad_set_state(rad_ctx* ctx, const float* radiosity, const float* illumination);

/* Copies Patch::radiosity and Patch::illumination (N*3 each; either may be NULL).  The
 * arrays must be writable host memory; pageable arrays have one byte per page read and
 * written back unchanged before the copy (it populates the pages), so a failed call leaves
 * their contents as they were. */
int rad_download(rad_ctx* ctx, float* radiosity, float* illumination);

/* precomputeHemicubeFormFactors (source/FormFactors.cpp:280-339): `copies` stacked
 * texture-layout tables, 2W x 1.5W floats each, written to out. */
int rad_ff_table(rad_ctx* ctx, float* out, uint32_t copies);

/* ModelContainer::getHighestRadiosityPatchesId (source/ModelContainer.cpp:259-299) on
 * the device-resident state: K ids and validity flags (valid[k]==0 <=> NULL emitter).
 * PHYS mode selects the K largest unshot powers instead. */
int rad_select_shooters(rad_ctx* ctx, uint32_t* ids, uint8_t* valid);

/* Hemicube item buffers of `count` shooters (the 5-face draw of source/Main.cpp:1155-1198):
 * count stacked 2W x 1.5W uint32 images, 0 = nothing, else patch index + 1. */
int rad_render_item_buffers(rad_ctx* ctx, const uint32_t* shooters, uint32_t count, uint32_t* items);

/* ProcessHemicube (source/Kernel_ProcessHemicube.h:9-70) plus the record accumulation
 * of source/Main.cpp:1257-1269 on caller-given item buffers: count x N form factors. */
int rad_reduce_item_buffers(rad_ctx* ctx, const uint32_t* items, uint32_t count, float* ff_rows);

/* Render + reduce fused: count x N form-factor rows of the given shooters. */
int rad_ff_rows(rad_ctx* ctx, const uint32_t* shooters, uint32_t count, float* ff_rows);

/* The hemicube cameras of `count` shooters (1..1024) as the draw uses them:
 * Camera::lookFromPatch (source/Camera.cpp:19-52) for the faces UP, DOWN, LEFT, RIGHT,
 * FRONT, each view matrix multiplied by Perspective(90, 1, 0.01, 1000)
 * (source/Main.cpp:1166-1184).  mvp receives count x 5 column-major 4x4 matrices; frames
 * (may be NULL) receives count x 6 floats, Patch::getCenter then Patch::getNormal
 * (source/Patch.cpp:261-276). */
int rad_face_cameras(rad_ctx* ctx, const uint32_t* shooters, uint32_t count, float* mvp, float* frames);

/* Runs up to n_shots batches of the shoot loop (source/Main.cpp:1137-1309) on the
 * device-resident state, K = hemicubes_count shooters per batch; stops early on the
 * stop rule.  stats may be NULL. */
int rad_shoot(rad_ctx* ctx, uint32_t n_shots, rad_stats* stats);

/* Stages of one shoot batch, in launch order (rad_profile_stages). */
#define RAD_STAGE_SELECT 0   /* shooter selection (1 kernel) */
#define RAD_STAGE_CAMERA 1   /* face MVPs + saved energy (1 kernel) */
#define RAD_STAGE_SETUP 2    /* raster record setup + bin counts (1 kernel) */
#define RAD_STAGE_BINS 3     /* bin scan + fill (2 kernels) */
#define RAD_STAGE_RASTER 4   /* tile raster + fused delta-FF reduction (1 kernel) */
#define RAD_STAGE_UPDATE 5   /* radiosity update (1 kernel) */
#define RAD_STAGE_EMITTERS 6 /* emitters + stop rule (1 kernel) */
#define RAD_N_STAGES 7

/* Diagnostic twin of rad_shoot: runs up to n_shots batches launched stage by stage
 * (no CUDA graph) with CUDA events between stages on the context stream and adds
 * each stage's device milliseconds to stage_ms[RAD_N_STAGES] (caller zeroes it).
 * The state advances exactly as with rad_shoot.  stats may be NULL. */
int rad_profile_stages(rad_ctx* ctx, uint32_t n_shots, double* stage_ms, rad_stats* stats);

/* Result of rad_autotune. */
typedef struct rad_tuning {
    uint32_t tile;             /* chosen raster bin side */
    uint32_t small_tri_pixels; /* chosen span/warp split */
    uint32_t hemicubes_count;  /* chosen K (unchanged unless RAD_TUNE_K) */
    uint32_t candidates;       /* configurations timed */
    double us_per_hemicube;    /* render + reduce time of the chosen configuration */
} rad_tuning;

#define RAD_TUNE_K 1u /* also choose K among 8..128 (changes the batching of the solve) */

/* Times the hemicube render + reduce pipeline on the current top shooters for each
 * candidate raster configuration (bin side 16/32/64 x span/warp split 64..4096 px,
 * optionally K) and reconfigures the context with the fastest.  The radiosity state is
 * not modified.  out may be NULL. */
int rad_autotune(rad_ctx* ctx, uint32_t flags, rad_tuning* out);

/* ---- Precision form: dense form factors and the gathering solve ---------------------
 * No counterpart in the reference (its solve is progressive shooting only): the rows of
 * the form-factor matrix are captured with the same hemicube pipeline (one hemicube per
 * patch), stored as BF16 with one FP32 scale per row (and optionally FP32), and
 * B = E + rho o (F B) is solved by mixed-precision iterative refinement: FP32 residuals,
 * BF16 Jacobi sweeps of the correction on tcgen05 tensor cores (FP32 accumulation),
 * FP64 norms.  rho is the scene's reflectance (PHYS mode). */
#define RAD_DENSE_FP32 1u /* also keep FP32 rows: needed by rad_gather_solve */
/* Shoot form: solve the fixed point of the progressive shooter instead,
 *     B_i = E_i + rho_i (sum_j F_ji A_j B_j) / A_i,
 * whose transfer j -> i is F_ji A_j / A_i: the reciprocity form the shoot update uses
 * (source/Main.cpp:1268-1276 with the area ratio of the PHYS rule).  The capture also keeps
 * the transposed rows (BF16, and FP32 with RAD_DENSE_FP32) and the area weights; the gather
 * then converges to the plain shooter's answer.  rad_gather_solve, rad_gather_residual and
 * the multi-scene graph use the form of the last capture; rad_dense_rows still returns rows
 * of F.  PHYS mode only. */
#define RAD_DENSE_SHOOT_FORM 2u

/* Captures every row of F (N hemicubes).  device_ms may be NULL. */
int rad_dense_capture(rad_ctx* ctx, uint32_t flags, double* device_ms);

/* Copies rows [first, first+count) of the captured matrix: FP32 (count x N), the BF16
 * bits (count x N) and the row scales (count); any output may be NULL. */
int rad_dense_rows(rad_ctx* ctx, uint32_t first, uint32_t count, float* f32, uint16_t* bf16, float* scale);

typedef struct rad_gather_stats {
    uint32_t outer;           /* FP32 residual evaluations */
    uint32_t sweeps;          /* BF16 tcgen05 sweeps */
    double initial_residual;  /* max over columns of ||r_c||_2 / ||E_c||_2 at the guess */
    double residual;          /* the same at return */
    double device_ms;         /* whole solve, CUDA events */
    double sweep_ms;          /* inside the tcgen05 sweeps */
    double resid_ms;          /* inside the FP32 residual GEMMs */
} rad_gather_stats;

/* Solves B = E + rho o (F B) for R <= 256 right-hand sides, column-major N x R host
 * arrays (column c uses reflectance channel c % 3).  guess may be NULL (start from E).
 * Stops when the relative residual <= tol or after max_outer refinements; each
 * refinement runs `sweeps` BF16 sweeps.  Needs rad_dense_capture(RAD_DENSE_FP32).
 * RAD_E_INVALID when emission or guess holds NaN / inf; RAD_E_NUMERIC when a residual norm
 * is not finite (radiosity then holds the last iterate). */
int rad_gather_solve(rad_ctx* ctx, const float* emission, uint32_t R, const float* guess, double tol,
                     uint32_t max_outer, uint32_t sweeps, float* radiosity, rad_gather_stats* stats);

/* r = E + rho o (F B) - B with the FP32 rows (column-major N x R host arrays); with B = E
 * this is the first-shot direct light rho o (F E).  In the shoot form F B is replaced by
 * (sum_j F_ji A_j B_j) / A_i, as in rad_shoot_residual. */
int rad_gather_residual(rad_ctx* ctx, const float* emission, uint32_t R, const float* radiosity, float* residual);

/* Residual of the system the progressive shooter solves, r_j = E_j + rho_j (sum_i F_ij A_i B_i)
 * / A_j - B_j (reciprocity form of the shoot update, source/Main.cpp:1268-1276), on the FP32
 * rows, same arrays as rad_gather_residual.  The two discretisations differ by the hemicube
 * reciprocity error, so each method is checked against its own system. */
int rad_shoot_residual(rad_ctx* ctx, const float* emission, uint32_t R, const float* radiosity, float* residual);

/* Self-test of the device-side failure path: a kernel waits on an mbarrier that nothing
 * completes, with the bound every pipeline wait of this library has (limit_us here, 2 s in
 * the solver kernels).  Returns RAD_E_TIMEOUT once the wait has given up and the kernel has
 * returned (the expected outcome), with the measured wall time in *waited_ms (may be NULL);
 * the device stays usable.  limit_us in 1..2,000,000. */
int rad_selftest_bounded_wait(int device, uint32_t limit_us, double* waited_ms);

/* Diagnostic: C = A * Bt^T on the tcgen05 path (A n x k, Bt R x k BF16 bits, row-major;
 * C column-major R x n FP32), on `device`. */
int rad_bf16_gemm(int device, const uint16_t* A, const uint16_t* Bt, uint32_t n, uint32_t k, uint32_t R, float* C);

/* ---- Learned warm start -------------------------------------------------------------
 * No counterpart in the reference.  A per-patch MLP, 32 -> 128 -> 128 -> 128 -> 128 -> 3
 * with ReLU, BF16 weights (FP32 master copy, Adam) and FP32 accumulation, trained and
 * evaluated by this library's own kernels.  Its prediction only seeds rad_gather_solve,
 * which still iterates to the same tolerance.  Rows of X are 32 features per patch, rows
 * of T / Y are 3 outputs; host arrays, row-major. */
typedef struct rad_mlp rad_mlp;
int rad_mlp_create(int device, uint64_t seed, rad_mlp** out);
int rad_mlp_destroy(rad_mlp* mlp);
uint32_t rad_mlp_param_count(void);
/* FP32 master parameters: per layer W[out][in] then b[out]. */
int rad_mlp_get_params(rad_mlp* mlp, float* params);
int rad_mlp_set_params(rad_mlp* mlp, const float* params);
int rad_mlp_predict(rad_mlp* mlp, const float* X, uint32_t P, float* Y);
/* Mean-squared-error loss of (X, T) and its gradient w.r.t. every parameter (no update). */
int rad_mlp_gradients(rad_mlp* mlp, const float* X, const float* T, uint32_t P, float* grads, double* loss);
/* Selects the engine of predict / gradients / train: on (the default) = tcgen05 tensor cores
 * (every layer a BF16 GEMM with FP32 accumulation in TMEM, activations and output gradients
 * rounded to BF16 between layers, bias / ReLU / ReLU-mask fused into the GEMM epilogues, weight
 * gradients by split-K GEMMs over the batch); off = CUDA cores with FP32 activations. */
int rad_mlp_set_tensor_cores(rad_mlp* mlp, int on);
/* Adam epochs over (X, T) in consecutive batches; the data set is copied to the device once. */
int rad_mlp_train(rad_mlp* mlp, const float* X, const float* T, uint32_t P, uint32_t epochs, uint32_t batch,
                  float lr, double* final_loss, double* device_ms);

/* ---- Many scenes under one CUDA graph ---------------------------------------------------
 * One graph replay advances every context by one shoot batch; the contexts' batches are
 * parallel branches of the graph, so scenes of uneven size share the GPU.  Contexts must
 * be on one device, have a scene uploaded, and must not be used elsewhere while the multi
 * object exists.  No counterpart in the reference (one scene per process). */
typedef struct rad_multi rad_multi;
int rad_multi_create(rad_ctx* const* ctxs, uint32_t count, rad_multi** out);
/* Replays up to n_replays times, stopping once every context's stop rule fired.
 * stop_replay[i] = replay index (1-based) after which context i had stopped, 0 if it never
 * did; stop_ms[i] = device time from the start of the call to the end of that replay
 * (may be NULL); *replays and *device_ms receive the totals. */
int rad_multi_shoot(rad_multi* m, uint32_t n_replays, uint32_t* stop_replay, double* stop_ms, uint32_t* replays,
                    double* device_ms);
int rad_multi_destroy(rad_multi* m);

/* ---- Many scenes solved by learned warm start + BF16 gather under one CUDA graph ----------
 * No counterpart in the reference.  Each context (PHYS mode, scene uploaded; its unshot
 * energy is the emission E) is a branch of one captured graph: dense capture of its form
 * factors (flags: 0 or RAD_DENSE_SHOOT_FORM, the system every branch solves), E and its
 * norms, the first-shot direct light rho o (F E), the network's 32 features
 * per patch and its guess (or, with mlp NULL, the guess E), the guess's residual, then the
 * refinements of rad_gather_solve (`sweeps` BF16 tcgen05 sweeps, update, FP32 residual with
 * FP64 norms) in a conditional loop that the device ends once the scene's relative residual
 * max_c ||r_c|| / ||E_c|| <= tol or after max_outer refinements.  feature_dirs: the 8 x 3
 * feature directions b_k of the sin / cos features (needed with an mlp).  Contexts must stay
 * alive and unused elsewhere while the object exists; their dense rows stay readable
 * (rad_dense_rows) after a run. */
typedef struct rad_multi_gather rad_multi_gather;
int rad_multi_gather_create(rad_ctx* const* ctxs, uint32_t count, const rad_mlp* mlp, const double* feature_dirs,
                            double tol, uint32_t max_outer, uint32_t sweeps, uint32_t flags,
                            rad_multi_gather** out);
/* One graph launch: every scene solved.  Per scene (arrays of count, any may be NULL): the
 * device ms from the graph's start to its final check, residual evaluations, final and
 * initial relative residual, status (1 converged, 2 stopped by max_outer, 3 non-finite);
 * *device_ms = the whole launch.  RAD_E_NUMERIC if a residual was not finite, RAD_E_TIMEOUT if
 * a pipeline wait gave up, RAD_E_OVERFLOW on raster capacity. */
int rad_multi_gather_run(rad_multi_gather* m, double* device_ms, double* scene_ms, uint32_t* outer,
                         double* residual, double* initial_residual, uint32_t* status);
/* Scene `index`'s radiosity after a run: 3 x N floats (channel-major, as rad_gather_solve). */
int rad_multi_gather_result(rad_multi_gather* m, uint32_t index, float* radiosity);
int rad_multi_gather_destroy(rad_multi_gather* m);

/* Raster counters of the last rad_profile_stages call (8 values): record-bin pairs (a record
 * holds both triangles of a patch quad), small records (row spans), their box pixels, big
 * records (one warp per triangle), their 8x4 stamps, stamps visited, stamps wholly inside,
 * big-triangle pixels written. */
int rad_raster_counters(rad_ctx* ctx, uint64_t* out);

/* Diagnostic twin of rad_profile_stages whose raster kernel also reads the SM clock at its
 * phase boundaries: runs up to n_shots batches (the state advances as with rad_shoot) and
 * writes the SM cycles the raster's warps spent per phase, summed over warps, to cycles[8]:
 * bin set-up, record staging, row ownership, row spans, pixel stream, pass barrier, big
 * records and chunk barrier, bin end (item buffer / reduction).  The clock reads slow the
 * raster down by about a fifth, so its stage times are not the kernel's.  stats may be NULL. */
int rad_profile_raster_phases(rad_ctx* ctx, uint32_t n_shots, uint64_t* cycles, rad_stats* stats);

/* Builds the reference scene (ModelContainer::load, source/ModelContainer.cpp:35-56,
 * PrimitiveModel ROOM/ROOMCLOSURE/CUBE/BLOCK subdivided to max_patch_area).  Call with
 * NULL arrays to get *n; then again with arrays of capacity >= *n patches. */
int rad_scene_reference(double max_patch_area, uint32_t capacity, uint32_t* n, float* vertices,
                        int32_t* indices, float* color, float* radiosity, float* illumination);

/* ---- Scene inputs, display output and checkpoints around the shoot loop --------------- */

/* The 8 display neighbours of every patch of the reference scene (N x 8 scene indices,
 * numbered from the upper left corner clockwise; a patch that was not divided is its own
 * neighbour): Patch::neighbours as set by Patch::divide (source/Patch.cpp:128-219) and
 * Model::subdivide (source/Model.cpp:38-46).  Same calling convention as rad_scene_reference. */
int rad_scene_reference_neighbours(double max_patch_area, uint32_t capacity, uint32_t* n, uint32_t* neighbours);

/* WaveFrontModel (source/WaveFrontModel.cpp:15-143) on an in-memory OBJ file of `length`
 * bytes, subdivided to max_patch_area (0 = not subdivided) as ModelContainer does: "v"
 * lines scaled by 1/1000, "f" lines with 3 or 4 vertices (a triangle repeats its last
 * vertex), other faces and faces naming a missing vertex skipped.  Patches are black with
 * no energy.  RAD_E_INVALID on a vertex line with fewer than 3 coordinates (the
 * reference's parse error).  Outputs as rad_scene_reference plus the neighbours (N x 8);
 * any array may be NULL; call with all NULL to get *n. */
int rad_scene_obj(const char* text, uint64_t length, double max_patch_area, uint32_t capacity, uint32_t* n,
                  float* vertices, int32_t* indices, float* color, float* radiosity, float* illumination,
                  uint32_t* neighbours);

/* .rr scene files of SaveToFile / LoadFromFile (source/Main.cpp:1460-1647,
 * source/LoadingModel.cpp:4-17): a 32-bit patch count, then the reference's Patch
 * objects as raw bytes (radiosity, illumination, relativeNeighbours[8], neighbours[8]
 * written as NULL pointers, the 4 corners, color), 148 bytes each from a 32-bit build
 * (pointer_bytes = 4) or 184 bytes from a 64-bit build (pointer_bytes = 8).  rad_rr_write
 * writes such a file into out (rad_rr_size bytes; neighbours may be NULL = each patch its
 * own); rad_rr_read detects the build from the file size and returns the scene (patches in
 * file order, not subdivided again, as LoadingModel) with *pointer_bytes; RAD_E_INVALID on
 * a size that fits neither build or a neighbour index out of range. */
int rad_rr_size(uint32_t n, uint32_t pointer_bytes, uint64_t* bytes);
int rad_rr_write(uint32_t n, const float* vertices, const float* color, const float* radiosity,
                 const float* illumination, const uint32_t* neighbours, uint32_t pointer_bytes, void* out,
                 uint64_t capacity);
int rad_rr_read(const void* data, uint64_t length, uint32_t capacity, uint32_t* n, float* vertices, int32_t* indices,
                float* color, float* radiosity, float* illumination, uint32_t* neighbours, uint32_t* pointer_bytes);

/* Uploads the scene's display neighbours (N x 8 patch indices, e.g. from
 * rad_scene_reference_neighbours / rad_scene_obj / rad_rr_read) for rad_display_colors. */
int rad_upload_neighbours(rad_ctx* ctx, const uint32_t* neighbours);

/* The display update after a batch of shots (source/Main.cpp:1318-1372) on the
 * device-resident state: colors = Colors::smoothShadePatch of every patch
 * (source/Colors.cpp:198-262; needs rad_upload_neighbours), radiative = each patch's
 * radiosity at its 4 corners; N x 12 floats each in the reference's VBO layout, either
 * may be NULL.  rad_display_colors copies them to host arrays; rad_display_colors_device
 * writes caller-owned device buffers (a headless stand-in for the mapped GL VBOs). */
int rad_display_colors(rad_ctx* ctx, float* colors, float* radiative);
int rad_display_colors_device(rad_ctx* ctx, float* d_colors, float* d_radiative);

/* ModelContainer::getHighestRadiosityPatchId (source/ModelContainer.cpp:222-237) on the
 * device-resident state: the first patch with the largest |radiosity|^2; PHYS mode: the
 * first with the largest unshot power (r+g+b)*area. */
int rad_highest_patch(rad_ctx* ctx, uint32_t* id);

/* Progress of the shoot loop for checkpoint / resume: batches done so far and the initial
 * unshot power that the PHYS residual is relative to (set by rad_upload_scene).  Restore
 * both after re-uploading a saved state so that the residual and stop rule continue. */
int rad_progress(rad_ctx* ctx, uint32_t* shots_done, double* initial_power);
int rad_set_progress(rad_ctx* ctx, uint32_t shots_done, double initial_power);

/* Allocation-free form-factor rows.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory (their device memory belongs to another
 * allocator's pool, or their loop must not allocate per call).  Inputs and outputs are
 * the caller's DEVICE buffers: d_items holds `count` stacked 2W x 1.5W uint32 item
 * buffers (0 = nothing, else patch index + 1; ids above n_patches are ignored) and
 * d_ff_rows receives count x n_patches floats, the same values rad_reduce_item_buffers
 * returns.  `stream` is a cudaStream_t (NULL = default stream); the call waits for the
 * stream to finish (cudaStreamSynchronize) before it returns.  No rad_ctx, no cudaMalloc/cudaFree: the only
 * scratch is a fixed device array of RAD_NOALLOC_MAX_SUMS 64-bit sums (8 MiB) that every
 * GPU loading the library holds until exit, so count * n_patches must not exceed
 * RAD_NOALLOC_MAX_SUMS (else RAD_E_NOALLOC_LIMIT).  The first call on a device looks the
 * array up; calls that overlap on the GPU race on the shared array. */
#define RAD_NOALLOC_MAX_SUMS (1u << 20)
int rad_reduce_items_noalloc(const uint32_t* d_items, uint32_t count, uint32_t hemicube_side,
                             uint32_t n_patches, float* d_ff_rows, void* stream);

const char* rad_strerror(int status);
const char* rad_last_error(const rad_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
