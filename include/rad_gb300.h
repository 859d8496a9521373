/*
 * rad_gb300.h -- C ABI of the GB300 progressive-refinement radiosity solver.
 *
 * Drop-in replacement for the shooting loop of morris821028/hw-radiosity.
 * The reference keeps its state in globals (TriStore[], trinum, G0, G1:
 * include/rad.h:51-55, src/rad.cpp:33-36) and calls, per shooter step,
 * listCanditate() -> Shade() -> AdaptCalFF()/CalFF() -> RayHitted()
 * (src/rad.cpp:387-451, src/shade.cpp:107-168, 435-462, src/raycast.cpp:335-360).
 * Here the host keeps the topology work (scene input, neighbour links,
 * pre-partition, output) and the device keeps the mesh, the visibility
 * structure and the unshot energy resident in HBM and runs the whole loop.
 *
 * Conventions: every call returns RAD_OK (0) or an RAD_ERR_* code and leaves a
 * one-line message for rad_last_error() (thread-local).  Handles are not
 * re-entrant: drive one handle from one host thread; separate handles are
 * independent.  Plain pointers and sizes only.
 */
#ifndef RAD_GB300_H
#define RAD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAD_OK 0
#define RAD_ERR_ARG 1        /* bad argument */
#define RAD_ERR_IO 2         /* file could not be opened or written */
#define RAD_ERR_PARSE 3      /* malformed .tri input (reference: assert in ReadVector/ReadIVector) */
#define RAD_ERR_CAPACITY 4   /* a size exceeds a stated limit */
#define RAD_ERR_CUDA 5       /* a CUDA runtime call failed */
#define RAD_ERR_WALK 6       /* a visibility walk hit its step cap (result for that ray: not visible) */
#define RAD_ERR_NODEV 7      /* no CUDA device */

/* Solver options: the reference's command-line globals (src/rad.cpp:17-31),
 * same names, meaning and defaults, plus two extensions at the end. */
typedef struct rad_options {
    int32_t debug;          /* -debug        Debug = 0 */
    float adapt_area;       /* -adapt_area   AreaLimit = 5.0 */
    float sample_area;      /* -sample_area  SampleArea = -1 (model dependent: max area / 100) */
    float converge;         /* -converge     ConvergeLimit = 1200.0 (absolute unshot key) */
    float delta_ff;         /* -delta_ff     DeltaFFLimit = 5e-6 */
    int32_t write_cycle;    /* -write_cycle  WriteIteration = 10 */
    int32_t zip;            /* -zip          CompressResult = 0 */
    int32_t triangle_limit; /* -triangle     TriangleLimit = 1000000 */
    float light_scale;      /* -light        LightScale = 1.0 */
    int32_t interactive;    /* -interactive  InteractiveOutput = 0 */
    int32_t jobs;           /* -jobs         host threads for host-side steps (default 2) */
    int32_t parallel_src;   /* -parallel_src ParallelSource = 1 (shooters per step) */
    /* extensions */
    int32_t precision;      /* 32: FP32 solver (reference FP32 build); 64: all-FP64 form */
    int32_t walk_cap;       /* max cell steps per visibility walk (default 65536; a walk of the
                               reference crosses at most a few hundred cells) */
} rad_options;

typedef struct rad_scene rad_scene;   /* host scene store */
typedef struct rad_octree rad_octree; /* host-built visibility structure */
typedef struct rad_dev rad_dev;       /* device-resident solver */
typedef struct rad_batch rad_batch;   /* many independent scenes shot together */
typedef struct rad_adapt rad_adapt;   /* the adaptive split variant */

/* Read-only view of a scene's live slots (valid until the scene changes or
 * is freed).  Arrays are slot-major; element type float (precision 32) or
 * double (precision 64) for the real-valued fields. */
typedef struct rad_scene_view {
    int32_t n;              /* live slots (trinum) */
    int32_t n_orig;         /* triangles read from the input */
    int32_t elem_size;      /* 4 or 8 */
    const void* p;          /* n*9  vertices p[3][3] */
    const void* accB;       /* n*9  accumulated radiosity per vertex and channel */
    const void* deltaB;     /* n*3  unshot radiosity per channel */
    const void* area;       /* n */
    const void* nrm;        /* n*3  unit normal */
    const void* ctr;        /* n*3  centre */
    const int32_t* parent;  /* n    original triangle id, -1 for a split (logical) slot */
    const int32_t* frgb;    /* n*3  reflectance 0..255 */
    const int32_t* brgb;    /* n*3  emission; a channel == 255 marks a light */
    const int32_t* nb;      /* n*3  neighbour across edge p0-p1, p1-p2, p2-p0 */
    float G0[3], G1[3];     /* grid corners (as float) */
    float sample_area;      /* resolved SampleArea */
    float min_area, max_area;
} rad_scene_view;

/* Statistics of a device run. */
typedef struct rad_stats {
    int64_t steps;          /* shooter steps executed (calls of parallelRadiosity that shot) */
    int64_t shots;          /* shooters processed (steps * shooters per step) */
    int64_t rays;           /* visibility walks issued */
    int64_t rays_ref;       /* walks the reference issues for the same work (adds the
                               whole-source walk AdaptCalFF discards, src/shade.cpp:141-168) */
    int64_t cells;          /* octree cells visited (0 unless counting is on) */
    int64_t tri_tests;      /* ray/triangle plane tests (0 unless counting is on) */
    int64_t se_tests;       /* edge-plane tests after a plane hit (0 unless counting is on) */
    int64_t prec_steps;     /* "Precision Exceeded" re-steps, src/raycast.cpp:344-351 */
    int64_t walk_cap_hits;  /* walks stopped by walk_cap */
    int32_t converged;      /* 1 once a selection found no candidate */
    int32_t n_slots;
    int64_t device_bytes;   /* device memory held by the handle */
    int64_t walk_loops;     /* walks stopped because their state repeated: the reference's
                               RayHitted never returns on these (ray treated as blocked) */
    double unshot_power;    /* sum over live slots of (dB_r + dB_g + dB_b) * area, reduced in
                               FP64 in a fixed order: the convergence monitor (rad_dev_stats
                               only; selection keeps the reference's FP32 key, rad.cpp:394) */
    int64_t h2d_bytes;      /* bytes copied host -> device when the handle was created */
} rad_stats;

void rad_options_default(rad_options* o);
const char* rad_last_error(void);
const char* rad_version(void);

/* ---- host scene store --------------------------------------------------- */

/* ReadTriangle, src/rad.cpp:47-111 (+ the "Read #Triangle" line of
 * InitModelFromFile, src/rad.cpp:244-252). */
int rad_scene_load(const char* path, const rad_options* o, rad_scene** out);
/* Same from arrays: vtx[n*9] (float), frgb[n*3], brgb[n*3]. */
int rad_scene_from_arrays(const float* vtx, const int32_t* frgb, const int32_t* brgb, int32_t n,
                          const rad_options* o, rad_scene** out);
/* InitRadiosity, src/rad.cpp:259-356: light energy, neighbour links
 * (exact-coordinate edge matching through a hash instead of the O(N^2) scan,
 * same final links as the sequential scan), SampleArea. */
int rad_scene_init(rad_scene* s);
/* The same with the neighbour links found on the device: every candidate
 * write of the reference's pair scan is made at once, the last one in the
 * scan's (i, j, v, n) order winning through a 64-bit atomicMax; the links
 * equal rad_scene_init's.  At most 2^20 triangles. */
int rad_scene_init_device(rad_scene* s, int32_t device);
/* PrePartitionTriangles, src/shade.cpp:556-598 (greedy longest-edge
 * bisection of the largest non-light triangles until area < 1 or the pool
 * is full). */
int rad_scene_prepartition(rad_scene* s);
int rad_scene_view_get(const rad_scene* s, rad_scene_view* v);
/* PrintOut, src/rad.cpp:117-242: prefix.fin (loop 0) or prefix.<loop>. */
int rad_scene_write_fin(const rad_scene* s, const char* prefix, int32_t loop);
/* Info lines (reference wording) produced by the last host-side call. */
const char* rad_scene_log(const rad_scene* s, int32_t stream); /* 1 = stdout lines, 2 = stderr lines */
void rad_scene_free(rad_scene* s);

/* ---- visibility structure ---------------------------------------------- */

/* BuildTree, src/raycast.cpp:168-233, over the scene's original triangles
 * (call before rad_scene_prepartition, as the reference does).  Reports the
 * reference's #TreeNode / #Trilist counts. */
int rad_octree_build(const rad_scene* s, int32_t threads, rad_octree** out);
/* The same tree with the triangle-box overlap tests on the device, level by
 * level (the host files the triangles into the children).  Leaves are
 * numbered level by level rather than depth first; every leaf's box and list,
 * the cell-to-leaf map up to that numbering, and the reference's counts are
 * those of rad_octree_build. */
int rad_octree_build_device(const rad_scene* s, int32_t device, rad_octree** out);
/* Copies of the flattened tree (sizes from rad_octree_info): the leaf of each
 * cell, dims[0]*dims[1]*dims[2]; per leaf its box (g0.xyz, 0, g1.xyz, 0 in
 * the octree's precision) and [begin, end) range; the triangle of each list
 * entry.  Any pointer may be null. */
int rad_octree_tables(const rad_octree* t, int32_t* cell_leaf, void* leaf_box, int32_t* leaf_range,
                      int32_t* entry_tri);
int rad_octree_info(const rad_octree* t, int64_t* ref_nodes, int64_t* ref_list, int32_t* n_leaves,
                    int64_t* n_entries, int32_t dims[3]);
/* Cell coordinates of points q[n] (float or double per the octree's
 * precision) on one axis, two ways: out_ref by the reference's expression
 * (int)(((double)q - G0) / MinGridLen) (raycast.cpp:263), out_fast by the
 * threshold search the device uses.  They are equal for q inside [G0, G1]. */
int rad_octree_cell_coords(const rad_octree* t, int32_t axis, const void* q, int32_t n, int32_t* out_ref,
                           int32_t* out_fast);
void rad_octree_free(rad_octree* t);

/* ---- device solver ------------------------------------------------------ */

/* Upload the scene (after init + pre-partition) and the visibility structure
 * to device `device`.  The walk's triangle records are taken from the
 * scene's current slots, as RayHitted reads TriStore at shooting time. */
int rad_dev_create(const rad_scene* s, const rad_octree* t, const rad_options* o, int32_t device, rad_dev** out);
/* Run up to max_steps shooter steps (parallelRadiosity, src/rad.cpp:406-451,
 * each: select -> shoot to every receiver -> zero the shooters).  Stops early
 * when a selection finds no candidate (*converged = 1).  Steps are issued in
 * CUDA-graph chunks; the host synchronises once per chunk. */
int rad_dev_run(rad_dev* d, int64_t max_steps, int64_t* steps_done, int32_t* converged);
/* The CUDA stream (a cudaStream_t) the handle's steps, downloads and queries
 * run on (no reference counterpart).  Work the caller enqueues there runs
 * before the steps of its next rad_dev_run* call, without a host round trip:
 * a timing loop that clears L2 between steps enqueues the clearing there. */
int rad_dev_stream(const rad_dev* d, void** stream);
/* rad_dev_run, also reporting the device time of the executed steps in
 * milliseconds (CUDA events on the solver's stream around the graph
 * launches; host synchronisation is outside the measured interval). */
int rad_dev_run_timed(rad_dev* d, int64_t max_steps, int64_t* steps_done, int32_t* converged, double* device_ms);
/* Steps one kernel launch at a time (no graph) with CUDA events around each
 * kernel: *ms_setup and *ms_shoot receive the summed durations of the
 * selection/setup kernel and the shooting kernel. */
int rad_dev_run_profiled(rad_dev* d, int64_t max_steps, int64_t* steps_done, int32_t* converged, double* ms_setup,
                         double* ms_shoot);
/* Copy accB and deltaB back into the scene's slots. */
int rad_dev_download(rad_dev* d, rad_scene* s);
/* Shooter ids chosen so far, in order (P per step; -1 pads a short step). */
int rad_dev_trace(const rad_dev* d, int32_t* out, int64_t cap, int64_t* n);
int rad_dev_stats(const rad_dev* d, rad_stats* st);
/* Count cells / triangle tests / edge tests during later steps (slower). */
/* The single-shooter schedule (no reference counterpart; results do not
 * depend on it).  A 10-slot group whose work item took longer than
 * max(split_frac * step time, split_mean_mult * mean group time) in one step
 * is shot in the next as 2-slot items with 4 lanes per corner; an item that
 * was already split stays split above split_frac_split * step time; a group
 * over early_mean_mult * mean group time is handed out first.  Defaults
 * 0.55, 0.27, 3.0, 1.5.  All zero splits every group after the first step
 * (tests use this to run the 4-lane walk everywhere); large values turn it
 * off. */
int rad_dev_set_schedule(rad_dev* d, double split_frac, double split_frac_split, double split_mean_mult,
                         double early_mean_mult);
int rad_dev_set_counting(rad_dev* d, int32_t on);
/* Which k_shoot form the single-shooter FP32 solver launches (no reference
 * counterpart; results do not depend on it).  1: 3 CTAs per SM, slow groups
 * split across 4 lanes per corner (for scenes whose step is bound by its
 * slowest groups).  2: 4 CTAs per SM, slow groups split into 3-slot items on
 * one lane each (for scenes with over 4 groups per resident warp, bound by
 * throughput).  0: choose by that rule, as the upload does.  Several shooters
 * per step, counting and FP64 always use form 1. */
int rad_dev_set_layout(rad_dev* d, int32_t layout);
/* The form chosen (1 or 2). */
int rad_dev_layout(const rad_dev* d);
/* Choose the form by timing both on this scene's own steps: one untimed step
 * in each form, then trials of steps_per_trial (1..32) steps in each form, in
 * alternating order, until max_steps steps have been shot or the solution
 * converged.  The faster form per step is kept (*chosen).  The steps are
 * ordinary solver steps (counted in *steps_done, traced, results unchanged);
 * a handle with one form (FP64, several shooters per step, counting) just
 * runs them. */
int rad_dev_autotune(rad_dev* d, int32_t steps_per_trial, int64_t max_steps, int64_t* steps_done,
                     int32_t* converged, int32_t* chosen);
/* Batched RayHitted (src/raycast.cpp:335-360): for each i, the triangle the
 * walk from p[i] along v[i] (not normalised) stops at, skipping ban[i]; -1 if
 * it leaves the grid.  Host arrays in and out (precision 32: float). */
int rad_dev_ray_hit(rad_dev* d, const void* p, const void* v, const int32_t* ban, int32_t n, int32_t* hit);
/* Batched Shade form factors without deposit: ff[i*3+v] for receiver slot
 * rcv[i] from shooter slot src (AdaptCalFF(CalFF(...)), src/shade.cpp:442-450). */
int rad_dev_form_factors(rad_dev* d, int32_t src, const int32_t* rcv, int32_t n, void* ff);
/* Form factors without allocating: the variant of rad_dev_form_factors for
 * callers that cannot call cudaMalloc or cudaFree when they call this -- a
 * renderer or simulation loop whose own allocator holds the whole device
 * memory budget, or a real-time loop that cannot take the implicit
 * synchronisation an allocation brings.  No counterpart in the reference
 * (its CalFF runs on host memory only).
 *   src    host array of n_src shooter slots, 1 <= n_src <= 64
 *   d_rcv  device array of n_rcv receiver slots (caller-allocated)
 *   d_ff   device array of n_src * n_rcv * 3 reals (float, or double for a
 *          precision-64 handle), caller-allocated; d_ff[(s*n_rcv + i)*3 + v]
 *          is corner v of receiver d_rcv[i] seen from shooter src[s], as
 *          rad_dev_form_factors computes it; a receiver slot outside the
 *          scene gives NaN
 *   stream cudaStream_t to enqueue on (NULL: the legacy default stream); the
 *          call returns without synchronising
 * The shooter records go to one fixed device array of 64 records (11 KB, held
 * by every GPU that loads the library until exit) instead of allocated
 * memory; more than 64 shooters is RAD_ERR_CAPACITY.  Every call reuses that
 * array, so calls whose kernels can overlap on the GPU (different streams
 * without ordering) race on it; order them on one stream.  The kernels also
 * add to the handle's walk counters, so finish or order `stream` before any
 * other call on the same handle.  The first call on each device looks the
 * array's device address up (cudaGetSymbolAddress with that device current)
 * and keeps it for the life of the process: make that first call before any
 * stream capture, and do not call again after cudaDeviceReset.  The caller's
 * current device is unchanged on return.  A walk stopped by walk_cap or by a
 * repeated state gives form factor 0 for that corner, as an occluded ray
 * does; such walks are counted only in the handle's rad_stats
 * (walk_cap_hits, walk_loops), not per call. */
int rad_dev_form_factors_noalloc(rad_dev* d, const int32_t* src, int32_t n_src, const int32_t* d_rcv, int32_t n_rcv,
                                 void* d_ff, void* stream);
void rad_dev_destroy(rad_dev* d);

/* ---- batched form -------------------------------------------------------- */

/* Upload n_scenes independent scenes (each after init + pre-partition, with
 * its own options: converge limit, walk cap) for the batched form: every
 * iteration, each scene that has not converged does one shooter step of
 * parallelRadiosity (src/rad.cpp:406-451), all scenes in one persistent
 * launch.  All scenes share one precision (32 or 64) and one -parallel_src P
 * (listCanditate's top n per scene, src/rad.cpp:387-404).  FP32 with P = 1
 * runs one kernel per iteration (the selection fused into its last CTA); FP64
 * or P > 1 adds a selection kernel, one CTA per scene.  Each scene's result is
 * bit-identical to rad_dev_run on that scene.  trace_cap: steps kept per
 * scene in its trace (P entries each; default 65536 when <= 0).  The octree
 * cells and list records are expanded on the device from the compact tables
 * (a leaf per cell, a triangle per list entry). */
int rad_batch_create(const rad_scene* const* scenes, const rad_octree* const* trees, const rad_options* opts,
                     int32_t n_scenes, int32_t trace_cap, int32_t device, rad_batch** out);
/* Run up to max_iters batch iterations; stops when every scene converged.
 * *iters_done: iterations in which at least one scene was running (a scene's
 * last iteration is the one whose selection finds no candidate);
 * *n_active: scenes still running. */
int rad_batch_run(rad_batch* b, int64_t max_iters, int64_t* iters_done, int32_t* n_active);
/* As rad_batch_run, also reporting the device time of the iterations (ms). */
int rad_batch_run_timed(rad_batch* b, int64_t max_iters, int64_t* iters_done, int32_t* n_active, double* device_ms);
int rad_batch_scene_stats(const rad_batch* b, int32_t scene, int64_t* steps, int32_t* converged);
int rad_batch_download(rad_batch* b, int32_t scene, rad_scene* s);
int rad_batch_trace(const rad_batch* b, int32_t scene, int32_t* out, int64_t cap, int64_t* n);
/* Totals over all scenes (steps = shooter steps of all scenes). */
int rad_batch_stats(const rad_batch* b, rad_stats* st);
int rad_batch_set_counting(rad_batch* b, int32_t on);
/* The shooting kernel's form (no reference counterpart; results do not depend
 * on it): 1 = 4 CTAs per SM (64 registers), 2 = 3 CTAs per SM (80 registers).
 * FP32 batches start in form 1, FP64 in form 2. */
int rad_batch_set_form(rad_batch* b, int32_t form);
int rad_batch_form(const rad_batch* b);
/* Choose the form by timing: one untimed iteration in each form, then
 * `rounds` rounds of iters_per_trial (1..32) iterations in each form, in
 * alternating order; the faster form per iteration is kept (*chosen).  The
 * iterations are ordinary batch iterations (results unchanged). */
int rad_batch_autotune(rad_batch* b, int32_t iters_per_trial, int32_t rounds, int32_t* chosen);
void rad_batch_destroy(rad_batch* b);

/* ---- adaptive split variant ---------------------------------------------- */

/* The reference built with include/config.h = ADAPT + ROLLBACK only:
 * serialRadiosity (rad.cpp:452-490) -- the first strict maximum shoots, and
 * receivers are visited in slot order -- with the full Shade
 * (shade.cpp:435-554): receivers of area >= adapt_area whose corner and centre
 * form factors (and up to area/sample_area rand() sample points) disagree by
 * more than delta_ff are split along the longest edge, with rollback.  Call
 * after rad_scene_init and WITHOUT rad_scene_prepartition (that configuration
 * has none).  The scene is updated in place by rad_adapt_run (topology,
 * accB, deltaB): write it with rad_scene_write_fin; it must outlive the
 * handle.  Each step's corner and centre form factors, the delta-FF test of
 * every receiver and the form factors of the sample points it draws are
 * computed on the device (the sample points speculatively, at the rand()
 * position they get if no earlier receiver breaks its sample loop); the
 * receiver loop in slot order, the splits with their neighbour links and
 * rollback, and every value whose inputs a split changed run on the host. */
int rad_adapt_create(rad_scene* s, const rad_octree* t, const rad_options* o, int32_t device, rad_adapt** out);
int rad_adapt_run(rad_adapt* a, int64_t max_steps, int64_t* steps_done, int32_t* converged);
int rad_adapt_trace(const rad_adapt* a, int32_t* out, int64_t cap, int64_t* n);
/* host_points: form factors evaluated on the host (sample points, receivers
 * rewritten earlier in their step); splits; rand() sample points drawn. */
int rad_adapt_stats(const rad_adapt* a, rad_stats* st, int64_t* host_points, int64_t* splits, int64_t* samples);
/* How the host takes the device's sample points (no reference counterpart;
 * results do not depend on it).  wait = 0 (the default): when a receiver's
 * sample loop moves the rand() stream off the speculation, a new speculation
 * starts at once from the next receiver, and the host takes each point the
 * device has already written and evaluates the others itself (fewer stalls,
 * more host form factors).  wait = 1: a new speculation starts when the next
 * sampling receiver needs it, and the host waits for it to finish (more
 * stalls, fewer host form factors). */
int rad_adapt_set_speculation(rad_adapt* a, int32_t wait);
/* The device's share (no reference counterpart): sample points whose form
 * factor came from the device's speculation, speculation launches, and
 * receivers whose delta-FF test failed at the start of their step (summed
 * over steps). */
int rad_adapt_device_stats(const rad_adapt* a, int64_t* device_points, int64_t* speculations,
                           int64_t* split_candidates);
void rad_adapt_destroy(rad_adapt* a);

/* ---------------------------------------------------------------- headless render
 * Replaces the reference's WebGL viewer path for a result: the model
 * converter (WebGL_demo/model-converter/main.cpp:167-246, JSON writer 81-150)
 * and the viewer's shaders in their initial state (WebGL_demo/public/index.html
 * drawScene 354-380, defaults 555-600; lib/flat.vs, flat.fs, gouraud.vs,
 * gouraud.fs), rasterised by CUDA kernels into an RGBA8 buffer, top row first.
 * No graphics API is used.  The reference has no C entry point for this; the
 * viewer runs in a browser on the converter's JSON. */
typedef struct rad_render_options {
    int32_t width, height;   /* pixels; default 1024 x 768 (the viewer's canvas), at most 16384 each */
    int32_t shading;         /* 0 flat (the viewer's default), 1 gouraud */
    int32_t pad;
    float x_rot, y_rot;      /* degrees, the viewer's eyeview.xRot / yRot; default 0 */
} rad_render_options;

void rad_render_options_default(rad_render_options* o);
/* render a .fin file (the reference's or ours); rgba holds width*height*4 bytes */
int rad_render_fin(const char* fin_path, const rad_render_options* o, int32_t device, uint8_t* rgba);
/* render a scene in memory: the triangles its .fin would hold */
int rad_render_scene(const rad_scene* s, const rad_render_options* o, int32_t device, uint8_t* rgba);

#ifdef __cplusplus
}
#endif
#endif
