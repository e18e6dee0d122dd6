/*
 * ppm_oracle.h -- CPU FP64 restatement of ppm-pa's data-parallel hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product path is compared against.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arm may load it.  Nothing in the
 * product (ppmpa_gb300/, include/) links to it.
 *
 * Parity pinning (what ties this restatement to the reference):
 *   - known-answer values from the reference's own unit tests:
 *       src/tracer.rs:369-376 (filter_cone / filter_gauss),
 *       src/ray/algebra.rs:268 (normalize), src/ray/geometry.rs:213-243
 *       (Ray::new_from_elem, target, get_normal), src/ray/physics.rs:374-377
 *       (Color::normalize, decide_wavelength), src/ray/physics.rs:408-416
 *       (check_under) -- see tests/test_oracle_kat.py;
 *   - the kd-tree demo points of src/bin/kdtreetest.rs:19-50 for the
 *     in-radius predicate;
 *   - the third-party `kdtree` crate (= "0.5.1", Cargo.toml:13, not vendored)
 *     is restated from its published algorithm: `within(p, r2, squared_euclidean)`
 *     returns every stored point whose f64 distance
 *     ((0 + dx*dx) + dy*dy) + dz*dz  (dx = query - point) is <= r2.
 *   The reference's random stream (`rand::thread_rng`, rand 0.6) cannot be
 *   seeded, so images are not pinned to reference outputs: the restatement
 *   replaces it with a seedable counter-based stream (Philox4x32-10) that
 *   makes the same number and order of draws per event as the reference.
 *
 * Struct layouts are identical to the public C ABI (include/ppm_api.h) so
 * one scene description feeds both; orc_sizeof() lets tests assert it.
 */
#ifndef PPM_ORACLE_H
#define PPM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shape kinds: src/ray/geometry.rs:66-90 */
enum { ORC_POINT = 0, ORC_PLAIN = 1, ORC_SPHERE = 2, ORC_POLYGON = 3, ORC_PARALLELOGRAM = 4 };
/* Surface kinds: src/ray/surface.rs:16-41 */
enum { ORC_NOTHING = 0, ORC_SIMPLE = 1, ORC_TS = 2 };
/* Light kinds: src/ray/light.rs:16-39 */
enum { ORC_LPOINT = 0, ORC_LPARALLELOGRAM = 1, ORC_LSUN = 2, ORC_LSPOT = 3 };
/* Photon filters: src/ray/optics.rs:17-21 */
enum { ORC_PF_NONE = 0, ORC_PF_CONE = 1, ORC_PF_GAUSS = 2 };

typedef struct orc_object {
    int32_t shape, material;
    double position[3], nvec[3], dir1[3], dir2[3];
    double dist, radius;
} orc_object;

typedef struct orc_material {
    double emittance[3], transmittance[3], ior[3];
    int32_t surface, pad_;
    double color_diff[3];   /* Simple.reflectance  | TS.albedo_diff */
    double color_spec[3];   /* Simple.specular_refl | TS.albedo_spec */
    double scatter;         /* Simple.diffuseness  | TS.scatterness */
    double metalness, roughness, density_pow, alpha;
} orc_material;

typedef struct orc_light {
    int32_t kind, pad_;
    double color[3], flux;
    double pos[3], nvec[3], dir1[3], dir2[3], dir[3];
} orc_light;

typedef struct orc_camera {
    int32_t xreso, yreso;
    int32_t progressive, antialias, blur, use_classic;
    int32_t pfilter, n_sample_photon;
    double radius, max_radiance, iso_sens, shut_speed, focal_len, f_number, focus;
    double ambient[3], eye_pos[3], target[3], upper[3];
    /* derived (orc_camera_derive) */
    double eye_dir[3], origin[3], esx[3], esy[3], eex[3], eey[3];
    double photon_power;
} orc_camera;

typedef struct orc_scene {
    const orc_object *objs;  int32_t n_objs;
    const orc_material *mats; int32_t n_mats;
    const orc_light *lights; int32_t n_lights;
} orc_scene;

int orc_sizeof(int which); /* 0 object, 1 material, 2 light, 3 camera */

/* math mode: 0 = own pm_* sin/cos/log/exp (bit-identical to the GPU FP64 path),
 *            1 = C library libm (closest to the reference's Rust f64 calls). */
void orc_set_libm(int on);
void orc_set_threads(int n);
int  orc_get_threads(void);

/* ---- scalar known-answer functions ------------------------------------ */
int    orc_normalize(const double *v, double *out);
double orc_filter_cone(double d, double rmax);
double orc_filter_gauss(double d, double rmax);
/* filter_gauss with an explicit CORR constant (tracer.rs:211 uses 0.5; the
 * reference's unit-test goldens at tracer.rs:374-376 correspond to 0.355,
 * the value left in the comment on that line). */
double orc_filter_gauss_corr(double d, double rmax, double corr);
int    orc_check_under(const double *ps, int n, double p);
void   orc_color_normalize(const double *c, double *out);
int    orc_decide_wavelength(const double *c, double p);
double orc_schlick(double f0, double cos);
double orc_relative_ior(double a, double b);
void   orc_ray_target(const double *pos, const double *dir, double t, double *out);
int    orc_new_dir(double x, double y, double z, double *out);
int    orc_get_normal(const orc_object *o, const double *p, double *out);
void   orc_material_derive(orc_material *m);
void   orc_camera_derive(orc_camera *c);
double orc_pm_sin(double x);
double orc_pm_cos(double x);
double orc_pm_exp(double x);
double orc_pm_log(double x);
void   orc_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out);

/* ---- deterministic kernels ---------------------------------------------- */
/* rays: n x 6 (pos, dir).  t[i] = nearest t >= NEARLY0, id[i] = object index
 * (-1 = miss); nrm (optional, n x 3) = oriented normal; io (optional) 1=In 0=Out. */
void orc_intersect(const orc_scene *sc, const double *rays, int64_t n,
                   double *t, int32_t *id, double *nrm, int32_t *io);

/* In-radius set: kdtree.within(q, r2, squared_euclidean) (src/tracer.rs:180).
 * Returns total neighbour count; fills offsets[nq+1] and idx[] (if idx != NULL
 * and total <= cap).  Indices per query in ascending photon index order. */
int64_t orc_within(const double *ppos, int64_t np, const double *q, int64_t nq,
                   const double *r2, int64_t *offsets, int32_t *idx, int64_t cap);

/* estimate_radiance (src/tracer.rs:179-195) per query: rgb[i] = sum over
 * neighbours in ascending distance order of photon_to_radiance(n, wt*pw, p),
 * times 1/(pi r2).  wl: 0 Red, 1 Green, 2 Blue. */
void orc_estimate(const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                  const double *qpos, const double *qnrm, int64_t nq,
                  double r2, double pw, int pfilter, double *rgb);

/* The same estimate with a radius per query (r2[i]), as the FP32 photon map's
 * estimate entry point takes them; one grid over the photons serves all. */
void orc_estimate_radii(const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                        const double *qpos, const double *qnrm, int64_t nq,
                        const double *r2, double pw, int pfilter, double *rgb);
/* wall seconds of the query phase (grid build excluded) of the last call above */
double orc_last_query_seconds(void);

/* Per query, the flux sums of estimate_radiance before its pw and 1/(pi r2)
 * factors: sums[3i + wl] = sum over the photons within r2, in ascending
 * distance, of wt(d, r2) * max(0, -n_i . dir); count[i] = photons within r2;
 * hash[i] = sum (mod 2^64) of SplitMix64's output function of
 * (index + 1) * 0x9e3779b97f4a7c15 over their indices (a set checksum). */
void orc_gather_sums(const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                     const double *qpos, const double *qnrm, int64_t nq, double r2, int pfilter,
                     int64_t *count, uint64_t *hash, double *sums);

/* ---- photon tracing (src/tracer.rs:31-125, src/ray/light.rs:67-91) ------ */
/* Emits the per-light counts of src/bin/ppmpa.rs:30-31 (pw = sum flux / nphoton,
 * n_l = round(flux_l / pw)) and traces every photon.  Stored photons are written
 * in emission order, deepest bounce first (the reference's push order).
 * Returns the number stored (or -needed if cap is too small). */
int64_t orc_trace_photons(const orc_scene *sc, int64_t nphoton, int uc, uint64_t seed,
                          uint32_t pass, double *pos, double *dir, uint8_t *wl,
                          int32_t *emit_idx, int8_t *level, int64_t cap,
                          double *power_out, int64_t *n_emitted_out);

/* One eye pass over a given photon map (src/bin/ppmpa.rs:81-82, src/tracer.rs:129-216):
 * image[3*pixel] += radiance of trace_ray for pixel (row-major). */
/* one pass of the classic (Whitted-style) tracer, trace_ray_classic
 * (tracer.rs:221-259) for every pixel's camera ray; adds into image. */
void orc_classic_pass(const orc_scene *sc, const orc_camera *cam, uint64_t seed, uint32_t pass, double *image);
void orc_eye_pass(const orc_scene *sc, const orc_camera *cam,
                  const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                  double r2, double pw, int uc, uint64_t seed, uint32_t pass, double *image);

/* Progressive render: passes of (trace photons, build map, eye pass) with the
 * PA schedule r2_{k+1} = r2_k * ((k+o)+alpha)/((k+o)+1) (o = 1 for
 * util/iterator.rb:33-38, 0 for util/radius.rb:13-17), averaged over passes
 * (util/averager.rb:66-69).  image = sum / passes. */
void orc_render(const orc_scene *sc, const orc_camera *cam, int64_t nphoton, int passes,
                double r0, double alpha, int schedule_offset, int uc, uint64_t seed,
                double *image);

/* PA schedule helper: r2[k] for k in [0, passes). */
void orc_radius_schedule(double r0, double alpha, int schedule_offset, int passes, double *r2);

#ifdef __cplusplus
}
#endif
#endif
