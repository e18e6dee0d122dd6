/*
 * ppm_api.h -- C ABI of the GB300-native ppm-pa hot path (libppmpa_gb300.so).
 *
 * Plain C: pointers, sizes and POD structs only; no CUDA or C++ types cross
 * the boundary.  Every entry point returns a ppm_status (0 = OK); the text
 * of the last error of a context is ppm_last_error(ctx).  Nothing throws.
 *
 * Each entry point names the reference interface it replaces (eijian/ppmpa,
 * paths relative to that project).  Host buffers are owned by the caller and
 * copied; device memory is owned by the context.  One context per host
 * thread; a context is not thread-safe.
 */
#ifndef PPM_API_H
#define PPM_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPM_API_VERSION 1

typedef enum ppm_status {
    PPM_OK = 0,
    PPM_ERR_INVALID_ARG = 1,
    PPM_ERR_OOM = 2,
    PPM_ERR_CAPACITY = 3,   /* a caller buffer or a device queue is too small */
    PPM_ERR_TIMEOUT = 4,
    PPM_ERR_CUDA = 5,
    PPM_ERR_NOT_READY = 6,  /* e.g. no scene, camera or photon map yet */
    PPM_ERR_NO_DEVICE = 7
} ppm_status;

/* ---- scene description (src/ray/geometry.rs, material.rs, surface.rs, light.rs) */

enum { PPM_SHAPE_POINT = 0, PPM_SHAPE_PLAIN = 1, PPM_SHAPE_SPHERE = 2,
       PPM_SHAPE_POLYGON = 3, PPM_SHAPE_PARALLELOGRAM = 4 };
enum { PPM_SURF_NOTHING = 0, PPM_SURF_SIMPLE = 1, PPM_SURF_TS = 2 };
enum { PPM_LIGHT_POINT = 0, PPM_LIGHT_PARALLELOGRAM = 1, PPM_LIGHT_SUN = 2, PPM_LIGHT_SPOT = 3 };
enum { PPM_FILTER_NONE = 0, PPM_FILTER_CONE = 1, PPM_FILTER_GAUSS = 2 };
enum { PPM_WL_RED = 0, PPM_WL_GREEN = 1, PPM_WL_BLUE = 2 };

/* Object = Shape + material index (src/ray/object.rs:10-13, geometry.rs:66-90).
 * Plain: infinite plane nvec.x + dist = 0.  Sphere: position = centre.
 * Polygon (triangle) / Parallelogram: position = p0, dir1 = p1-p0, dir2 = p2-p0,
 * nvec = normalize(dir1 x dir2). */
typedef struct ppm_object {
    int32_t shape;
    int32_t material;
    double position[3];
    double nvec[3];
    double dir1[3];
    double dir2[3];
    double dist;
    double radius;
} ppm_object;

/* Material + Surface (src/ray/material.rs:11-16, surface.rs:16-41).
 * Simple: color_diff = reflectance, color_spec = specular_refl, scatter = diffuseness.
 * TS:     color_diff = albedo_diff, color_spec = albedo_spec, scatter = scatterness.
 * density_pow and alpha are derived: call ppm_material_derive(). */
typedef struct ppm_material {
    double emittance[3];
    double transmittance[3];
    double ior[3];
    int32_t surface;
    int32_t pad_;
    double color_diff[3];
    double color_spec[3];
    double scatter;
    double metalness;
    double roughness;
    double density_pow;
    double alpha;
} ppm_material;

/* Light (src/ray/light.rs:16-39).  color is used as given: the reference's
 * scene code normalises it (Color::normalize) before building the light.
 * PPM_LIGHT_SPOT has no reference counterpart: a point light at pos whose
 * photons leave uniformly over the cone around the unit axis dir with
 * cos(half-angle) = dir1[0]; like the reference's point light it adds no
 * direct light (one sample, see get_radiance_from_light). */
typedef struct ppm_light {
    int32_t kind;
    int32_t pad_;
    double color[3];
    double flux;
    double pos[3];
    double nvec[3];
    double dir1[3];
    double dir2[3];
    double dir[3];
} ppm_light;

/* Camera (src/camera.rs:23-49).  The first block is read_camera's input
 * (camera.rs:108-146; focal_len in metres); the second block is derived by
 * ppm_camera_derive() exactly as camera.rs:150-175. */
typedef struct ppm_camera {
    int32_t xreso, yreso;
    int32_t progressive, antialias, blur, use_classic;
    int32_t pfilter, n_sample_photon;
    double radius, max_radiance, iso_sens, shut_speed, focal_len, f_number, focus;
    double ambient[3], eye_pos[3], target[3], upper[3];
    double eye_dir[3], origin[3], esx[3], esy[3], eex[3], eey[3];
    double photon_power;
} ppm_camera;

/* Progressive render configuration (src/bin/ppmpa.rs:15-84 plus the pass loop,
 * PA radius schedule and average of util/iterator.rb:33-38, util/averager.rb). */
enum { PPM_PRECISION_PLAIN = 0,   /* FP64 everywhere (reference semantics) */
       PPM_PRECISION_MIXED = 1 }; /* FP32 trace/gather + Kahan; FP64 radius, average, normalisation */

typedef struct ppm_render_cfg {
    int64_t nphoton;          /* photons per pass (#photon of ppmpa.rs:15) */
    int32_t passes;
    int32_t use_classic;      /* 1 = default, 0 = "-nc" (ppmpa.rs:50-54) */
    double radius0;           /* initial estimate radius (not squared) */
    double alpha;             /* PA alpha (iterator.rb:17 uses 0.5) */
    int32_t schedule_offset;  /* 1: iterator.rb:33-38; 0: radius.rb / averager.rb */
    int32_t precision;        /* PPM_PRECISION_* */
    int32_t use_graph;        /* capture one pass as a CUDA graph and replay it */
    int32_t cell_factor;      /* grid cells per radius (1 to 4; 0 = auto) */
    uint64_t seed;
    int32_t first_pass;       /* index of the first pass (for sharded/resumed runs) */
    int32_t flags;            /* PPM_RENDER_* bits; others must be 0 */
} ppm_render_cfg;

/* Render flags.  PPM_RENDER_TUNE_CELLS: pick the photon-map cells per radius
 * (1 to 4) by timing one trial pass with each before the render starts; the
 * trial passes leave no trace in the image.  No reference counterpart. */
enum { PPM_RENDER_TUNE_CELLS = 1,
/* PPM_RENDER_CLASSIC: the reference's classic ray tracer trace_ray_classic
 * (src/tracer.rs:221-259, the `rtc` binary) instead of photon mapping: each
 * pass traces the eye rays only (direct light + ambient, mirror and
 * refraction children); passes average anti-aliased images. */
       PPM_RENDER_CLASSIC = 2,
/* PPM_RENDER_TILE_GATHER: in the mixed render, gather with one warp per 32
 * hit points (one lane each, sorted into a compact patch of the scene,
 * sharing one walk of the photons around them) in place of the default row
 * walk (one warp per hit point, or per two in one cell, walking its own
 * cell rows).  Same neighbour sets and sums.  The tile form costs fewer
 * instructions per photon test but tests more photons (the union of 32
 * spheres against each sphere); which is faster depends on how dense the
 * hit points are beside the radius.  No reference counterpart. */
       PPM_RENDER_TILE_GATHER = 4 };

/* Per-pass statistics of the last rendered pass and accumulated timings. */
typedef struct ppm_stats {
    int64_t photons_emitted;   /* last pass */
    int64_t photons_stored;    /* last pass */
    int64_t hit_points;        /* last pass */
    int64_t grid_cells;        /* last pass */
    int64_t passes_done;
    int32_t kernels_per_pass;  /* CUDA kernels launched by one pass */
    int32_t n_stages;
    double  r2;                /* radius^2 of the last pass */
    double  stage_ms[16];      /* summed device time per stage (timing on) */
    int64_t stage_calls[16];
    int64_t candidates;        /* photons tested by the gather (last pass, stage timing level 2) */
    int64_t in_radius;         /* photons found in radius (last pass, stage timing level 2) */
    int64_t gather_slots;      /* lane slots the gather issued (last pass, stage timing level 2) */
    int32_t cell_factor;       /* grid cells per radius the render uses (tuned or given) */
    int64_t photon_rays;       /* photon ray segments traced (emission + bounces), last pass */
    int64_t eye_rays;          /* eye-tree rays traced (primary + reflected/refracted children;
                                  shadow rays not counted), last pass */
} ppm_stats;

typedef struct ppm_ctx ppm_ctx;

/* ---- context ----------------------------------------------------------- */
int         ppm_version(void);
const char *ppm_status_string(int status);
int         ppm_ctx_create(ppm_ctx **out, int device, uint64_t seed);
int         ppm_ctx_destroy(ppm_ctx *ctx);
const char *ppm_last_error(const ppm_ctx *ctx);
void       *ppm_ctx_stream(ppm_ctx *ctx);               /* the cudaStream_t all work runs on */
int         ppm_ctx_sync(ppm_ctx *ctx);

/* ---- scene and camera input ---------------------------------------------- */
/* Replaces read_scene (src/scene.rs:20): the scene arrives as data. */
int  ppm_scene_upload(ppm_ctx *ctx, const ppm_object *objs, int32_t n_objs,
                      const ppm_material *mats, int32_t n_mats,
                      const ppm_light *lights, int32_t n_lights);
/* Replaces read_camera (src/camera.rs:108): derives, then stores. */
int  ppm_camera_set(ppm_ctx *ctx, const ppm_camera *cam);
/* Scene and camera files.  The reference ships example/*.scene and *.scr
 * files (camera grammar: doc/ebnf-camera.txt) but its read_scene and
 * read_camera ignore them (src/scene.rs:20, src/camera.rs:108); these
 * readers turn the files into the structs above.  ppm_scene_parse: on input
 * *n_objs, *n_mats, *n_lights are the capacities of the arrays; with all
 * three arrays NULL it only counts.  ppm_camera_parse overrides the fields
 * the file sets (start from the reference camera) and derives the rest;
 * *nphoton gets the file's nphoton if present.  A syntax error, an unknown
 * type or name returns PPM_ERR_INVALID_ARG; ppm_parse_error() says where. */
int ppm_scene_parse(const char *text, ppm_object *objs, int32_t *n_objs, ppm_material *mats, int32_t *n_mats,
                    ppm_light *lights, int32_t *n_lights);
int ppm_camera_parse(const char *text, ppm_camera *cam, int64_t *nphoton);
const char *ppm_parse_error(void);

/* Ray acceleration.  The reference tests every object per ray
 * (tracer.rs:321-329).  From 32 bounded objects (spheres, triangles,
 * parallelograms) up, scene upload builds a BVH on the GPU and rays walk it;
 * results are the same (nearest t, then lowest index).  PPM_ACCEL_BVH forces
 * the hierarchy from 2 objects, PPM_ACCEL_NONE the loop; applies at once. */
enum { PPM_ACCEL_AUTO = 0, PPM_ACCEL_BVH = 1, PPM_ACCEL_NONE = 2 };
int  ppm_set_accel(ppm_ctx *ctx, int32_t mode);
/* objects per BVH leaf (1..8, default 1; leaves are runs of the Morton-ordered
 * objects); rebuilds the tree at once.  No reference counterpart. */
int  ppm_set_bvh_leaf(ppm_ctx *ctx, int32_t leaf_max);
/* Leaf-size autotuner: builds the tree with 1, 2, 4 and 8 objects per leaf,
 * times the FP32 first-hit kernel over the given rays (n x 6) and keeps the
 * fastest; returns it and its time.  No reference counterpart. */
int  ppm_tune_bvh_leaf(ppm_ctx *ctx, const double *rays, int64_t n, int32_t *best_leaf, double *best_ms);
/* objects in the hierarchy (0: none) and unbounded objects tested per ray */
int  ppm_accel_info(ppm_ctx *ctx, int32_t *bvh_objects, int32_t *unbounded);
/* Host helpers: camera.rs:150-175 and Surface::new_simple/new_ts (surface.rs:45-66). */
void ppm_camera_derive(ppm_camera *cam);
void ppm_material_derive(ppm_material *mat);

/* ---- FP64 parity entry points (host buffers) ------------------------------ */
/* calc_intersection (src/tracer.rs:306-350) for n rays (n x 6: pos, dir):
 * t[i] = nearest distance >= NEARLY0, obj[i] = object index or -1; nrm
 * (optional, n x 3) the normal oriented against the ray. */
int ppm_intersect(ppm_ctx *ctx, const double *rays, int64_t n,
                  double *t, int32_t *obj, double *nrm);
/* FP32 traversal of the same rays (the mixed-precision intersector). */
int ppm_intersect_f32(ppm_ctx *ctx, const double *rays, int64_t n,
                      double *t, int32_t *obj);

/* Photon emission + trace_photon for one pass (src/bin/ppmpa.rs:30-31, :86-92;
 * src/tracer.rs:31-125; src/ray/light.rs:67-91) in FP64.  Results stay on the
 * device; ppm_photons_download copies them out (order unspecified; emit_idx
 * and level identify each photon).  pass selects the random stream. */
int ppm_trace_photons(ppm_ctx *ctx, int64_t nphoton, int32_t use_classic, uint32_t pass,
                      int64_t *n_stored, double *power, int64_t *n_emitted);
int ppm_photons_download(ppm_ctx *ctx, double *pos, double *dir, uint8_t *wl,
                         int32_t *emit_idx, int8_t *level, int64_t cap);

/* build_photonmap (src/photonmap.rs:23-29): sort-by-cell grid over the given
 * photons (n x 3 positions / directions, wl 0..2), power pw, radius^2 r2. */
int ppm_photonmap_build(ppm_ctx *ctx, const double *pos, const double *dir,
                        const uint8_t *wl, int64_t n, double power, double radius2);
/* Build the map from the photons of the last ppm_trace_photons call. */
int ppm_photonmap_from_trace(ppm_ctx *ctx, double radius2);

/* kdtree.within(q, r2, squared_euclidean) (src/tracer.rs:180) per query with
 * its own r2[i] <= the map's radius2.  offsets has nq+1 entries; idx receives
 * photon indices (input order of ppm_photonmap_build), ascending per query.
 * idx == NULL: sizes only.  *total = sum of neighbour counts. */
int ppm_query_within(ppm_ctx *ctx, const double *q, int64_t nq, const double *r2,
                     int64_t *offsets, int32_t *idx, int64_t cap, int64_t *total);

/* estimate_radiance (src/tracer.rs:179-195): rgb (nq x 3) at positions with
 * oriented normals, using the map's power and radius2 and filter pfilter. */
int ppm_estimate(ppm_ctx *ctx, const double *pos, const double *nrm, int64_t nq,
                 int32_t pfilter, double *rgb);

/* ppm_estimate_noalloc: no counterpart in the reference.  Same arguments and
 * results as ppm_estimate, for at most PPM_ESTIMATE_NOALLOC_MAX_QUERIES
 * queries per call (more returns PPM_ERR_INVALID_ARG with a message), but it
 * never allocates or frees device memory.  It is for callers that cannot
 * let the library allocate mid-run: a host whose own memory pool already
 * holds nearly all of the device, or one that cannot take the device-wide
 * wait a cudaFree implies while its other streams run.  The queries and
 * results are staged in one fixed device array (about 5 MB) per device,
 * shared by every context and call in the process and held until the
 * process exits.  ppm_ctx_create places that array on its device and looks
 * up its address, so the entry point itself loads and allocates nothing;
 * a context created after a device reset looks it up again.  Calls whose
 * GPU work overlaps (two host threads, or two contexts on the same device)
 * race on the array: serialise them. */
#define PPM_ESTIMATE_NOALLOC_MAX_QUERIES 32768
int ppm_estimate_noalloc(ppm_ctx *ctx, const double *pos, const double *nrm, int64_t nq,
                         int32_t pfilter, double *rgb);

/* One eye pass over the FP64 map of ppm_photonmap_build, as the reference's
 * `rt` renders a map read from `pm` (src/bin/rt.rs:41-46): trace_ray
 * (tracer.rs:129-177) for every pixel with the map's power and radius^2;
 * pass selects the random streams.  image_out: yreso x xreso x 3. */
int ppm_eye_pass(ppm_ctx *ctx, int32_t use_classic, uint64_t seed, int32_t pass, double *image_out);

/* ---- FP32 photon map (gather sweep) --------------------------------------- */
/* A map of FP32 photons (n x 3 float positions, directions, wl).  Queries are
 * FP32 positions with FP64 radii^2; membership is decided exactly as the f64
 * predicate on the f32 values (FP32 test + FP64 recheck in the rounding band). */
int ppm_photonmap_build_f32(ppm_ctx *ctx, const float *pos, const float *dir,
                            const uint8_t *wl, int64_t n, double power, double radius2_max);
int ppm_query_within_f32(ppm_ctx *ctx, const float *q, int64_t nq, const double *r2,
                         int64_t *offsets, int32_t *idx, int64_t cap, int64_t *total);
/* Queries are gathered in the map's cell order on the device; rgb comes back
 * in the caller's order. */
int ppm_estimate_f32(ppm_ctx *ctx, const float *pos, const float *nrm, int64_t nq,
                     const double *r2, double *rgb);
/* Grid cell size of the FP32 map: cells_per_radius cells per maximum query
 * radius (default 2, range [0.5, 8]).  Re-sorts the map on the device; sets
 * and estimates do not change, only their cost.  No reference counterpart
 * (the reference's kd-tree has no cell size). */
int ppm_photonmap_regrid_f32(ppm_ctx *ctx, double cells_per_radius);
/* Autotuner: times sort + gather of a sample of queries with 1, 1.5, 2, 3
 * and 4 cells per radius, leaves the map on the fastest grid and returns it
 * (best_cells) with its device time in ms (best_ms).  No reference counterpart. */
int ppm_photonmap_tune_f32(ppm_ctx *ctx, const float *pos, const float *nrm, int64_t nq,
                           const double *r2, double *best_cells, double *best_ms);

/* ---- progressive render ---------------------------------------------------- */
/* Runs cfg->passes passes (emit + trace photons, build the map, eye trace,
 * gather, PA radius shrink, FP64 running sum) and writes the averaged image
 * (yreso x xreso x 3 doubles, row-major) -- the output of ppmpa (ppmpa.rs:36-41)
 * averaged as util/averager.rb:66-69. */
int ppm_render(ppm_ctx *ctx, const ppm_render_cfg *cfg, double *image_out);

/* Device-resident stepping: begin sets up buffers, resets the running sum and
 * the radius; step enqueues npasses passes on the context stream (async);
 * image averages the passes done so far. */
int ppm_render_begin(ppm_ctx *ctx, const ppm_render_cfg *cfg);
int ppm_render_step(ppm_ctx *ctx, int32_t npasses);
int ppm_render_image(ppm_ctx *ctx, double *image_out);
int ppm_render_pass_image(ppm_ctx *ctx, double *image_out);  /* the last pass alone */
int ppm_render_stats(ppm_ctx *ctx, ppm_stats *out);
/* on = 1: record per-stage CUDA events inside every pass (passes then run
 * eagerly, not as a graph); on = 2: also count gather candidates and hits. */
int ppm_set_stage_timing(ppm_ctx *ctx, int32_t on);
const char *ppm_stage_name(int32_t stage);

/* Parity export of the mixed-precision render's gather.  No reference
 * counterpart: it exposes, hit point by hit point, what the render's own
 * gather computes, so that it can be checked against estimate_radiance
 * (src/tracer.rs:179-216).  The call runs one more pass of the render begun
 * by ppm_render_begin (precision PPM_PRECISION_MIXED, photon mapping),
 * eagerly and counted like ppm_render_step(ctx, 1), in which the gather also
 * records per hit point: the FP32 flux sums per wavelength,
 *   sum over the photons p in radius of max(0, -n . dir_p) * wt(d2, r2),
 * before the hit point's weight and the pass's pw / (pi r2) scale them; the
 * number of photons in radius; and a checksum of that set, the sum (mod 2^64)
 * over their slots s in the pass's sorted photon map of SplitMix64's output
 * function of (s + 1) * 0x9e3779b97f4a7c15.  It copies out that pass's sorted
 * photon map (x, y, z, then the direction word: 15 + 15-bit octahedral
 * direction, wavelength in bits 30-31), its hit points and its FP32
 * gathered-flux image.  With photons == NULL it sets n_photons and n_hits to
 * the most one pass can produce and runs nothing. */
typedef struct ppm_gather_export {
    int64_t photon_cap, hit_cap;    /* in: entries the arrays below hold */
    int64_t n_photons, n_hits;      /* out */
    double radius2, photon_power;   /* out: the pass's r^2 and photon power pw */
    int32_t pass, pfilter;          /* out: the pass index and the camera's filter */
    float *photons;                 /* n_photons x 4: x, y, z, direction word (float bits) */
    float *hits;                    /* n_hits x 10: position, normal, weight, pixel (int32 bits) */
    float *sums;                    /* n_hits x 3 */
    uint32_t *counts;               /* n_hits */
    uint64_t *checksums;            /* n_hits */
    float *gathered;                /* yreso x xreso x 3: per pixel, sum of weight x sums */
} ppm_gather_export;
int ppm_render_gather_export(ppm_ctx *ctx, ppm_gather_export *ex);

/* ---- output ------------------------------------------------------------------ */
/* Camera::radiance_to_rgb (src/camera.rs:92-100) for n values:
 * floor(min(1, L / max_radiance)^(1/2.2) * 255); the averager's P3 output
 * (util/averager.rb:66-76) is this map of the averaged image. */
int ppm_tone_map(const double *img, int64_t n, double max_radiance, int32_t *rgb_out);
/* The uncompressed scanline OpenEXR file of util/averager2.rb:154-218 (B, G,
 * R float channels) with values img * scale; averager2 divides the averaged
 * image by max radiance (scale = 1 / max_radiance). */
int ppm_write_exr(const char *path, const double *img, int32_t xreso, int32_t yreso, double scale);

/* ---- batched rendering ------------------------------------------------------ */
/* No reference counterpart (the reference renders one scene per process,
 * one pass per run).  A batch renders many independent jobs -- scenes of any
 * size, cameras, photon budgets, alphas, pass counts -- on one GPU: each job
 * has its own context and captured pass graph, and every pass of the whole
 * batch is a single graph launch whose branches are the jobs, so small jobs
 * share the GPU instead of running one after another.  Jobs whose passes are
 * done drop out.  Each job's image is the same as ppm_render would give for
 * it alone (up to the order of floating-point atomic adds).  device_ms
 * (optional) receives the device time of all the passes. */
typedef struct ppm_job {
    const ppm_object *objs;
    int32_t n_objs;
    int32_t n_mats;
    const ppm_material *mats;
    const ppm_light *lights;
    int32_t n_lights;
    int32_t pad_;
    const ppm_camera *cam;
    ppm_render_cfg cfg;       /* use_graph is forced on */
    double *image_out;        /* yreso x xreso x 3 */
} ppm_job;

typedef struct ppm_batch ppm_batch;
int         ppm_batch_create(ppm_batch **out, int device, uint64_t seed);
int         ppm_batch_destroy(ppm_batch *b);
const char *ppm_batch_last_error(const ppm_batch *b);
int         ppm_batch_render(ppm_batch *b, const ppm_job *jobs, int32_t njobs, double *device_ms);

/* How a batch runs its passes.  PPM_BATCH_STAGED: one launch per stage of the
 * pass (eye levels, photon trace, map build, gather, accumulate) covers every
 * job -- 22 launches per pass whatever the number of jobs, each stage taking
 * its work items (job, element) from the concatenation of the jobs' work --
 * for 1 to 256 jobs that are all mixed-precision photon-mapping renders with
 * the default gather.  PPM_BATCH_GRAPHS: each job's own pass graph, the
 * jobs' graphs side by side in one parent graph per pass (any jobs).
 * PPM_BATCH_AUTO (default): when the jobs allow staged passes, the first
 * render times one pass of each mode on its jobs (the staged one after the
 * tile tuner) and keeps the faster for this and later renders, until the
 * next ppm_batch_set_mode; otherwise graphs.  tile: photons per work item of
 * the staged map-build stages; 0 (default) times 1024, 4096 and 16384 on one
 * pass of the batch before the render and keeps the fastest.
 * No reference counterpart. */
enum { PPM_BATCH_AUTO = 0, PPM_BATCH_STAGED = 1, PPM_BATCH_GRAPHS = 2 };
int         ppm_batch_set_mode(ppm_batch *b, int32_t mode, int32_t tile);
/* how the last render ran: staged (1) or graphs (0), and the tile it used */
int         ppm_batch_info(const ppm_batch *b, int32_t *staged, int32_t *tile);
/* AUTO's trial: ms per pass of the staged and graph modes it measured
 * (PPM_ERR_NOT_READY before the first AUTO render of staged-capable jobs) */
int         ppm_batch_trial_ms(const ppm_batch *b, double *staged_ms, double *graphs_ms);

#ifdef __cplusplus
}
#endif
#endif /* PPM_API_H */
