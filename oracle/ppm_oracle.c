/*
 * ppm_oracle.c -- CPU FP64 restatement of ppm-pa's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; never the product).  See
 * ppm_oracle.h for what pins it to the reference.  Every function below
 * cites the reference file:line it restates.  Arithmetic is IEEE f64 with
 * FMA contraction disabled (-ffp-contract=off) and evaluation order matching
 * the reference's Rust expressions, so that:
 *   - scalar results equal the reference's unit-test goldens, and
 *   - in own-math mode the photon paths are bit-identical to the GPU FP64
 *     path given the same seed (same draws, same rounding).
 *
 * Random stream (replaces rand::thread_rng, which cannot be seeded):
 *   Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 *   easy as 1, 2, 3", SC'11), key = 64-bit seed, counter =
 *   {item, pass, tag, block}.  Draw k of an event uses block k/2, 64-bit word
 *   k%2; u = (word >> 12) * 2^-52 (rand 0.6's 52-bit float construction) and
 *   gen_range(lo, hi) = u * (hi - lo) + lo.
 *   tags: EMIT (photon emission), BOUNCE|level (photon event at a level),
 *   CAMERA (eye ray jitter), EYE|node (eye vertex; root node 1, reflect
 *   child 2n, refract child 2n+1).
 */
#include "ppm_oracle.h"

#include <math.h>
#include <time.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NEARLY0 0.0001                 /* src/ray/mod.rs:16 */
#define MAX_TRACE 10                   /* src/tracer.rs:27 */
#define PI_D 0x1.921fb54442d18p+1
#define PI2_D (PI_D * 2.0)             /* src/ray/mod.rs:17 */
#define PI4_D (PI_D * 4.0)             /* src/ray/mod.rs:18 */
#define ONE_PI (1.0 / PI_D)            /* src/tracer.rs:24 */
#define SR_HALF (1.0 / (2.0 * PI_D))   /* src/tracer.rs:25 */
#define K_CONE 1.1                     /* src/tracer.rs:198 */
#define FAC_K (1.0 - 2.0 / (3.0 * K_CONE))
#define G_ALPHA 0.918                  /* src/tracer.rs:208-211 */
#define G_BETA 1.953
#define G_E_BETA (1.0 - 0.14184788965323)
#define G_CORR 0.5
#define PARA_DIV 0.2                   /* src/ray/light.rs:162 */

#define TAG_EMIT   0x01000000u
#define TAG_BOUNCE 0x02000000u
#define TAG_CAMERA 0x03000000u
#define TAG_EYE    0x04000000u

static int g_libm = 0;
static int g_threads = 0;

void orc_set_libm(int on) { g_libm = on; }
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_sizeof(int which) {
    switch (which) {
    case 0: return (int)sizeof(orc_object);
    case 1: return (int)sizeof(orc_material);
    case 2: return (int)sizeof(orc_light);
    case 3: return (int)sizeof(orc_camera);
    default: return -1;
    }
}

/* ------------------------------------------------------------------------ */
/* own f64 elementary functions (identical operation sequence on the GPU)   */
/* sin/cos: Cody-Waite reduction by pi/2 (three 33-bit chunks), Taylor      */
/* polynomials on |r| <= pi/4.  exp: reduction by ln2 (40-bit high part),   */
/* Taylor to r^14.  log: m in [sqrt(1/2), sqrt(2)], 2*atanh((m-1)/(m+1))   */
/* series to s^25.  Coefficients are 1/k! and 1/(2k+1) rounded to double.   */
/* ------------------------------------------------------------------------ */
static const double PIO2_1 = 0x1.921fb54400000p+0;
static const double PIO2_2 = 0x1.0b4611a600000p-34;
static const double PIO2_3 = 0x1.3198a2e037073p-69;
static const double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
static const double LN2_HI = 0x1.62e42fefa2000p-1;
static const double LN2_LO = 0x1.9ef35793c7673p-41;
static const double INV_LN2 = 0x1.71547652b82fep+0;
static const double SQRT2_D = 0x1.6a09e667f3bcdp+0;

static double bits2d(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t d2bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }

static void pm_sincos_r(double x, double *s, double *c) {
    double fk = floor(x * TWO_OVER_PI + 0.5);
    double r = ((x - fk * PIO2_1) - fk * PIO2_2) - fk * PIO2_3;
    double r2 = r * r;
    double ps = -0x1.2f49b46814157p-57;
    ps = ps * r2 + 0x1.952c77030ad4ap-49;
    ps = ps * r2 + -0x1.ae7f3e733b81fp-41;
    ps = ps * r2 + 0x1.6124613a86d09p-33;
    ps = ps * r2 + -0x1.ae64567f544e4p-26;
    ps = ps * r2 + 0x1.71de3a556c734p-19;
    ps = ps * r2 + -0x1.a01a01a01a01ap-13;
    ps = ps * r2 + 0x1.1111111111111p-7;
    ps = ps * r2 + -0x1.5555555555555p-3;
    double sr = r + (r * r2) * ps;
    double pc = 0x1.e542ba4020225p-62;
    pc = pc * r2 + -0x1.6827863b97d97p-53;
    pc = pc * r2 + 0x1.ae7f3e733b81fp-45;
    pc = pc * r2 + -0x1.93974a8c07c9dp-37;
    pc = pc * r2 + 0x1.1eed8eff8d898p-29;
    pc = pc * r2 + -0x1.27e4fb7789f5cp-22;
    pc = pc * r2 + 0x1.a01a01a01a01ap-16;
    pc = pc * r2 + -0x1.6c16c16c16c17p-10;
    pc = pc * r2 + 0x1.5555555555555p-5;
    pc = pc * r2 + -0x1.0000000000000p-1;
    double cr = 1.0 + r2 * pc;
    int q = (int)(((int64_t)fk) & 3);
    switch (q) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}

double orc_pm_sin(double x) { double s, c; pm_sincos_r(x, &s, &c); return s; }
double orc_pm_cos(double x) { double s, c; pm_sincos_r(x, &s, &c); return c; }

static double pm_scale2(double p, int k) {
    if (k > 1023) { p = p * bits2d((uint64_t)(1023 + 1023) << 52); k -= 1023; }
    if (k < -1022) { p = p * bits2d((uint64_t)(-1000 + 1023) << 52); k += 1000; }
    if (k < -1022) { p = p * bits2d((uint64_t)(-1000 + 1023) << 52); k += 1000; }
    return p * bits2d((uint64_t)(k + 1023) << 52);
}

double orc_pm_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    double fk = floor(x * INV_LN2 + 0.5);
    double r = (x - fk * LN2_HI) - fk * LN2_LO;
    double p = 0x1.93974a8c07c9dp-37;
    p = p * r + 0x1.6124613a86d09p-33;
    p = p * r + 0x1.1eed8eff8d898p-29;
    p = p * r + 0x1.ae64567f544e4p-26;
    p = p * r + 0x1.27e4fb7789f5cp-22;
    p = p * r + 0x1.71de3a556c734p-19;
    p = p * r + 0x1.a01a01a01a01ap-16;
    p = p * r + 0x1.a01a01a01a01ap-13;
    p = p * r + 0x1.6c16c16c16c17p-10;
    p = p * r + 0x1.1111111111111p-7;
    p = p * r + 0x1.5555555555555p-5;
    p = p * r + 0x1.5555555555555p-3;
    p = p * r + 0x1.0000000000000p-1;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return pm_scale2(p, (int)fk);
}

double orc_pm_log(double x) {
    if (x != x || x < 0.0) return NAN;
    if (x == 0.0) return -INFINITY;
    if (x == INFINITY) return x;
    uint64_t b = d2bits(x);
    int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) {
        x = x * 0x1p54;
        b = d2bits(x);
        e = (int)((b >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    double m = bits2d((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > SQRT2_D) { m = m * 0.5; e += 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double p = 0x1.47ae147ae147bp-5;
    p = p * s2 + 0x1.642c8590b2164p-5;
    p = p * s2 + 0x1.8618618618618p-5;
    p = p * s2 + 0x1.af286bca1af28p-5;
    p = p * s2 + 0x1.e1e1e1e1e1e1ep-5;
    p = p * s2 + 0x1.1111111111111p-4;
    p = p * s2 + 0x1.3b13b13b13b14p-4;
    p = p * s2 + 0x1.745d1745d1746p-4;
    p = p * s2 + 0x1.c71c71c71c71cp-4;
    p = p * s2 + 0x1.2492492492492p-3;
    p = p * s2 + 0x1.999999999999ap-3;
    p = p * s2 + 0x1.5555555555555p-2;
    double t = 2.0 * s;
    double lm = t + t * (s2 * p);
    double fe = (double)e;
    return (fe * LN2_LO + lm) + fe * LN2_HI;
}

static double m_sin(double x) { return g_libm ? sin(x) : orc_pm_sin(x); }
static double m_cos(double x) { return g_libm ? cos(x) : orc_pm_cos(x); }
static double m_exp(double x) { return g_libm ? exp(x) : orc_pm_exp(x); }
/* x^y for x >= 0 (the reference's powf on a uniform draw) */
static double m_pow(double x, double y) {
    if (g_libm) return pow(x, y);
    if (y == 0.0) return 1.0;
    if (x != x || y != y) return NAN;
    if (x == 0.0) return y > 0.0 ? 0.0 : INFINITY;
    if (x == 1.0) return 1.0;
    return orc_pm_exp(y * orc_pm_log(x));
}
/* x^5 (Schlick's (1-cos)^5, src/ray/physics.rs:317, src/ray/surface.rs:513) */
static double m_pow5(double x) {
    if (g_libm) return pow(x, 5.0);
    double x2 = x * x;
    double x4 = x2 * x2;
    return x4 * x;
}
/* x^2 (src/ray/algebra.rs:229) */
static double m_sq(double x) { return g_libm ? pow(x, 2.0) : x * x; }

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 counter-based stream                                       */
/* ------------------------------------------------------------------------ */
void orc_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int i = 0; i < 10; i++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct {
    uint32_t key[2], ctr[4];
    uint32_t buf[4];
    int k;
} rng_t;

static void rng_init(rng_t *r, uint64_t seed, uint32_t item, uint32_t pass, uint32_t tag) {
    r->key[0] = (uint32_t)seed; r->key[1] = (uint32_t)(seed >> 32);
    r->ctr[0] = item; r->ctr[1] = pass; r->ctr[2] = tag; r->ctr[3] = 0;
    r->k = 0;
}

/* next uniform in [0, 1) with 52 random bits */
static double rng_u(rng_t *r) {
    int w = r->k & 1;
    if (w == 0) {
        r->ctr[3] = (uint32_t)(r->k >> 1);
        orc_philox(r->ctr, r->key, r->buf);
    }
    uint64_t v = (uint64_t)r->buf[2 * w] | ((uint64_t)r->buf[2 * w + 1] << 32);
    r->k++;
    return (double)(v >> 12) * 0x1p-52;
}

/* rand 0.6 Rng::gen_range(lo, hi) for f64: value0_1 * scale + low */
static double gen_range(rng_t *r, double lo, double hi) {
    double u = rng_u(r);
    return u * (hi - lo) + lo;
}

/* ------------------------------------------------------------------------ */
/* Vector3 (src/ray/algebra.rs:22-196)                                      */
/* ------------------------------------------------------------------------ */
typedef struct { double x, y, z; } V3;
static inline V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static inline V3 v3p(const double *p) { V3 r = {p[0], p[1], p[2]}; return r; }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 vmul(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 smul(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline V3 vneg(V3 a) { return v3(-a.x, -a.y, -a.z); }
static inline double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 vcross(V3 a, V3 b) {
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline int vnormalize(V3 a, V3 *out) {
    double n = sqrt(vdot(a, a));
    if (n == 0.0) return 0;
    *out = vmul(a, 1.0 / n);
    return 1;
}

int orc_normalize(const double *v, double *out) {
    V3 r;
    if (!vnormalize(v3p(v), &r)) return 0;
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
    return 1;
}

int orc_new_dir(double x, double y, double z, double *out) {
    double v[3] = {x, y, z};
    return orc_normalize(v, out);
}

/* src/ray/geometry.rs:56-58 */
void orc_ray_target(const double *pos, const double *dir, double t, double *out) {
    V3 p = vadd(v3p(pos), vmul(v3p(dir), t));
    out[0] = p.x; out[1] = p.y; out[2] = p.z;
}

/* ------------------------------------------------------------------------ */
/* Colour / physics (src/ray/physics.rs)                                    */
/* ------------------------------------------------------------------------ */
/* Color::normalize, physics.rs:61-71 */
void orc_color_normalize(const double *c, double *out) {
    double r1 = c[0] < 0.0 ? 0.0 : c[0];
    double g1 = c[1] < 0.0 ? 0.0 : c[1];
    double b1 = c[2] < 0.0 ? 0.0 : c[2];
    double mag = r1 + g1 + b1;
    if (mag == 0.0) {
        out[0] = out[1] = out[2] = 1.0 / 3.0;
    } else {
        out[0] = r1 / mag; out[1] = g1 / mag; out[2] = b1 / mag;
    }
}

/* Color::decide_wavelength, physics.rs:74-84 */
int orc_decide_wavelength(const double *c, double p) {
    if (p < c[0]) return 0;
    if (p < c[0] + c[1]) return 1;
    return 2;
}

/* relative_ior, physics.rs:200-205 */
double orc_relative_ior(double a, double b) { return a == 0.0 ? 1.0 : b / a; }

static double relative_ior_average(const double *i1, const double *i2) {
    double a1 = (i1[0] + i1[1] + i1[2]) / 3.0;   /* physics.rs:192-196 */
    double a2 = (i2[0] + i2[1] + i2[2]) / 3.0;
    return orc_relative_ior(a1, a2);
}

/* schlick, physics.rs:316-318 */
double orc_schlick(double f0, double cos) { return f0 + (1.0 - f0) * m_pow5(1.0 - cos); }

/* check_under, physics.rs:329-335 */
int orc_check_under(const double *ps, int n, double p) {
    int i = 0;
    while (i < n && p > ps[i]) i++;
    return i;
}

/* russian_roulette with one threshold, physics.rs:323-327 */
static int rr1(rng_t *r, double p0) {
    double p = gen_range(r, 0.0, 1.0);
    return p > p0 ? 1 : 0;
}

/* specular_reflection, physics.rs:214-221 */
static V3 specular_reflection(V3 n, V3 v, double *cos_out) {
    double cos = -vdot(v, n);
    if (cos < 0.0) { *cos_out = -cos; return n; }
    V3 r;
    vnormalize(vadd(v, smul(2.0 * cos, n)), &r);
    *cos_out = cos;
    return r;
}

/* specular_refraction, physics.rs:270-285.  Returns 1 if a direction exists. */
static int specular_refraction(V3 n, V3 v, double eta, V3 *t_out, double *cos2) {
    double cos1 = -vdot(v, n);
    if (cos1 < 0.0) { *cos2 = 0.0; return 0; }
    double sq_eta = eta * eta;
    double sq_cos = cos1 * cos1;
    double g0 = sq_eta + sq_cos - 1.0;
    /* eta = 0: the reference's g / eta is 0/0 or x/0 where rounding makes
     * |cos1| reach 1 (NaN weights); no refraction, as the GPU paths */
    if (g0 < 0.0 || eta == 0.0) { *cos2 = 0.0; return 0; }
    double g = sqrt(g0);
    *cos2 = g / eta;
    return vnormalize(smul(1.0 / eta, vadd(v, smul(cos1 - g, n))), t_out);
}

/* reflection_glossy, physics.rs:232-261 (two draws) */
static V3 reflection_glossy(rng_t *rg, V3 n, V3 r, double pw) {
    V3 u = {1.0, 0.0, 0.0};
    if (!vnormalize(vcross(v3(0.00424, 1.0, 0.00764), r), &u))
        vnormalize(vcross(v3(1.0, 0.00424, 0.00764), r), &u);
    V3 v = vcross(u, r);
    double c0 = vdot(n, r);
    if (c0 < 0.0) c0 = 0.0;   /* rounding at grazing incidence; NaN below otherwise (as the GPU paths) */
    double xi0 = gen_range(rg, 0.0, 1.0);
    double xi1 = m_pow(xi0, pw * c0);
    double xi2 = 2.0 * PI_D * gen_range(rg, 0.0, 1.0);
    double sq = sqrt(1.0 - xi1 * xi1);
    double x = m_cos(xi2) * sq;
    double y = xi1;
    double z = m_sin(xi2) * sq;
    V3 wi = vadd(vadd(smul(x, u), smul(y, r)), smul(z, v));
    if (vdot(n, wi) < 0.0) wi = vsub(vadd(smul(-x, u), smul(y, r)), smul(z, v));
    V3 out;
    if (!vnormalize(wi, &out)) out = v3(1.0, 0.0, 0.0);
    return out;
}

/* generate_random_dir_by_angle, algebra.rs:225-235 (two draws) */
static V3 random_dir_by_angle(rng_t *rg) {
    double phi = gen_range(rg, 0.0, 2.0 * PI_D);
    double xi = gen_range(rg, -1.0, 1.0);
    double xi2 = sqrt(1.0 - m_sq(xi));
    V3 v = v3(xi2 * m_cos(phi), xi, xi2 * m_sin(phi)), out = {0.0, 1.0, 0.0};
    vnormalize(v, &out);
    return out;
}

/* diffuse_reflection, surface.rs:408-417 */
static V3 diffuse_reflection(rng_t *rg, V3 n) {
    V3 d = random_dir_by_angle(rg);
    return vdot(n, d) > 0.0 ? d : vneg(d);
}

/* generate_random_dir, algebra.rs:211-223 (3 draws per trial; the reference
 * loops unboundedly, this stops after 256 trials (p < 1e-80) with +y). */
static V3 random_dir(rng_t *rg) {
    for (int it = 0; it < 256; it++) {
        double x = gen_range(rg, -1.0, 1.0);
        double y = gen_range(rg, -1.0, 1.0);
        double z = gen_range(rg, -1.0, 1.0);
        V3 v = v3(x, y, z);
        double len = sqrt(vdot(v, v));
        if (0.0 < len && len <= 1.0) { V3 o; vnormalize(v, &o); return o; }
    }
    return v3(0.0, 1.0, 0.0);
}

/* ------------------------------------------------------------------------ */
/* Materials / surfaces (src/ray/surface.rs, material.rs)                   */
/* ------------------------------------------------------------------------ */
static const orc_material M_AIR = {    /* src/scene.rs:13-18 */
    {0, 0, 0}, {1, 1, 1}, {1, 1, 1}, ORC_NOTHING, 0, {0, 0, 0}, {0, 0, 0}, 0, 0, 0, 0, 0};

/* Surface::new_simple / new_ts derived fields, surface.rs:45-66 */
void orc_material_derive(orc_material *m) {
    m->density_pow = 1.0 / (pow(10.0, 5.0 * (1.0 - sqrt(m->roughness))) + 1.0);
    m->alpha = m->surface == ORC_TS ? m->roughness * m->roughness * m->roughness * m->roughness : 0.0;
}

static int col_eq(const double *c, double v) { return c[0] == v && c[1] == v && c[2] == v; }

/* Surface::reflect, surface.rs:68-100 */
static int sf_reflect(const orc_material *m, double cos) {
    if (m->surface == ORC_SIMPLE)
        return !(m->scatter == 1.0 || (cos == 1.0 && col_eq(m->color_spec, 0.0)));
    if (m->surface == ORC_TS) {
        if (m->metalness == 0.0) return 1;
        if (m->metalness == 1.0) return !col_eq(m->color_spec, 0.0);
        return 1;
    }
    return 0;
}

/* Surface::refract, surface.rs:102-133 */
static int sf_refract(const orc_material *m, double cos) {
    if (m->surface == ORC_SIMPLE) return !(cos == 0.0 && col_eq(m->color_spec, 1.0));
    if (m->surface == ORC_TS)
        return m->metalness == 0.0 && m->scatter < 1.0 && !col_eq(m->color_diff, 0.0);
    return 0;
}

/* Surface::store_photon, surface.rs:289-310 */
static int sf_store(const orc_material *m) {
    if (m->surface == ORC_SIMPLE) return m->scatter > 0.0;
    if (m->surface == ORC_TS) return m->metalness != 1.0 && m->scatter != 0.0;
    return 1;
}
static double sf_albedo_diff(const orc_material *m, int wl) {   /* surface.rs:312-333 */
    return (m->surface == ORC_SIMPLE || m->surface == ORC_TS) ? m->color_diff[wl] : 0.0;
}
static double sf_albedo_spec(const orc_material *m, int wl) {   /* surface.rs:335-356 */
    return (m->surface == ORC_SIMPLE || m->surface == ORC_TS) ? m->color_spec[wl] : 0.0;
}
static double sf_roughness(const orc_material *m) {            /* surface.rs:358-379 */
    if (m->surface == ORC_SIMPLE) return m->scatter;
    if (m->surface == ORC_TS) return m->roughness;
    return 0.0;
}
static double sf_power_glossy(const orc_material *m) {         /* surface.rs:381-402 */
    return (m->surface == ORC_SIMPLE || m->surface == ORC_TS) ? m->density_pow : 0.0;
}

/* reflection_index, surface.rs:512-515 */
static V3 reflection_index(const double *col, double c) {
    double c2 = m_pow5(1.0 - c);
    return v3(col[0] + (1.0 - col[0]) * c2, col[1] + (1.0 - col[1]) * c2, col[2] + (1.0 - col[2]) * c2);
}

/* Surface::bsdf, surface.rs:135-206, literal Radiance arithmetic order */
static V3 sf_bsdf(const orc_material *m, double cos0, V3 di, V3 si, V3 ti) {
    if (m->surface == ORC_SIMPLE) {
        V3 f = reflection_index(m->color_spec, cos0);
        V3 f2 = v3(1.0 - f.x, 1.0 - f.y, 1.0 - f.z);
        double d = m->scatter;
        V3 rp = v3(m->color_diff[0] * ONE_PI, m->color_diff[1] * ONE_PI, m->color_diff[2] * ONE_PI);
        V3 a = smul(d, v3(rp.x * di.x, rp.y * di.y, rp.z * di.z));
        double om = 1.0 - m->metalness;
        V3 fm = smul(om, f2);
        V3 inner = vadd(v3(f.x * si.x, f.y * si.y, f.z * si.z), v3(fm.x * ti.x, fm.y * ti.y, fm.z * ti.z));
        return vadd(a, smul(1.0 - d, inner));
    }
    if (m->surface == ORC_TS) {
        V3 f = reflection_index(m->color_spec, cos0);
        V3 f2 = v3(1.0 - f.x, 1.0 - f.y, 1.0 - f.z);
        V3 ide = v3(0, 0, 0);
        if (m->metalness == 0.0) {
            V3 fa = v3(f2.x * m->color_diff[0], f2.y * m->color_diff[1], f2.z * m->color_diff[2]);
            double sp = m->scatter * ONE_PI;
            V3 in = vadd(smul(sp, di), smul(1.0 - m->scatter, ti));
            ide = v3(fa.x * in.x, fa.y * in.y, fa.z * in.z);
        }
        V3 imt = v3(f.x * si.x, f.y * si.y, f.z * si.z);
        return vadd(ide, imt);
    }
    return v3(0, 0, 0);
}

/* ------------------------------------------------------------------------ */
/* Geometry (src/ray/geometry.rs:117-202) and calc_intersection             */
/* (src/tracer.rs:306-350)                                                  */
/* ------------------------------------------------------------------------ */
static int method_moller(double l, V3 p0, V3 d1, V3 d2, V3 p, V3 d, double *t) {
    V3 re2 = vcross(d, d2);
    double det_a = vdot(re2, d1);
    V3 pp = vsub(p, p0);
    V3 te1 = vcross(pp, d1);
    double u = vdot(re2, pp) / det_a;
    double v = vdot(te1, d) / det_a;
    double tt = vdot(te1, d2) / det_a;
    if (det_a == 0.0 || u < 0.0 || u > 1.0 || v < 0.0 || v > 1.0 || u + v > l) return 0;
    *t = tt;
    return 1;
}

static int shape_distance(const orc_object *o, V3 rp, V3 rd, double ts[2]) {
    switch (o->shape) {
    case ORC_PLAIN: {
        V3 n = v3p(o->nvec);
        double cos0 = vdot(n, rd);
        if (cos0 == 0.0) return 0;
        ts[0] = (o->dist + vdot(n, rp)) / -cos0;
        return 1;
    }
    case ORC_SPHERE: {
        V3 oc = vsub(v3p(o->position), rp);
        double t0 = vdot(oc, rd);
        double t1 = o->radius * o->radius - (vdot(oc, oc) - t0 * t0);
        double t2 = sqrt(t1);
        if (t1 <= 0.0) return 0;
        if (t2 == 0.0) { ts[0] = t0; return 1; }
        ts[0] = t0 - t2; ts[1] = t0 + t2;
        return 2;
    }
    case ORC_POLYGON:
    case ORC_PARALLELOGRAM: {
        double l = o->shape == ORC_POLYGON ? 1.0 : 2.0;
        return method_moller(l, v3p(o->position), v3p(o->dir1), v3p(o->dir2), rp, rd, &ts[0]);
    }
    default:
        return 0;
    }
}

int orc_get_normal(const orc_object *o, const double *p, double *out) {
    V3 n;
    switch (o->shape) {
    case ORC_PLAIN: case ORC_POLYGON: case ORC_PARALLELOGRAM:
        n = v3p(o->nvec); break;
    case ORC_SPHERE:
        if (!vnormalize(vsub(v3p(p), v3p(o->position)), &n)) return 0;
        break;
    default:
        return 0;
    }
    out[0] = n.x; out[1] = n.y; out[2] = n.z;
    return 1;
}

typedef struct { V3 pos, n; int obj, in; double t; } isect_t;

static int intersect(const orc_scene *sc, V3 rp, V3 rd, isect_t *is) {
    double best = 0.0;
    int bi = -1;
    for (int i = 0; i < sc->n_objs; i++) {
        double ts[2];
        int k = shape_distance(&sc->objs[i], rp, rd, ts);
        for (int j = 0; j < k; j++) {
            double t = ts[j];
            if (!(t >= NEARLY0)) continue;     /* t < NEARLY0 discarded (NaN too) */
            if (bi < 0 || t < best) { best = t; bi = i; }
        }
    }
    if (bi < 0) return 0;
    V3 p = vadd(rp, vmul(rd, best));
    double nn[3], pp[3] = {p.x, p.y, p.z};
    if (!orc_get_normal(&sc->objs[bi], pp, nn)) return 0;
    V3 n = v3p(nn);
    if (vdot(n, rd) > 0.0) { is->n = vneg(n); is->in = 0; }
    else { is->n = n; is->in = 1; }
    is->pos = p; is->obj = bi; is->t = best;
    return 1;
}

void orc_intersect(const orc_scene *sc, const double *rays, int64_t n,
                   double *t, int32_t *id, double *nrm, int32_t *io) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t i = 0; i < n; i++) {
        isect_t is;
        const double *r = rays + 6 * i;
        if (intersect(sc, v3p(r), v3p(r + 3), &is)) {
            t[i] = is.t; id[i] = is.obj;
            if (nrm) { nrm[3 * i] = is.n.x; nrm[3 * i + 1] = is.n.y; nrm[3 * i + 2] = is.n.z; }
            if (io) io[i] = is.in;
        } else {
            t[i] = 0.0; id[i] = -1;
            if (nrm) nrm[3 * i] = nrm[3 * i + 1] = nrm[3 * i + 2] = 0.0;
            if (io) io[i] = -1;
        }
    }
}

static const orc_material *mat_of(const orc_scene *sc, int m) { return m < 0 ? &M_AIR : &sc->mats[m]; }

/* ------------------------------------------------------------------------ */
/* Photon emission and tracing                                              */
/* ------------------------------------------------------------------------ */
typedef struct { int wl; V3 pos, dir; } photon_t;

/* Spot light: an extension with no reference counterpart (light.rs:16-38
 * has point, parallelogram and sun lights).  A point light whose photons
 * leave uniformly over the solid angle of the cone around the unit axis
 * l->dir with cos(half-angle) l->dir1[0]: u -> cos(theta) = 1 - u (1 - cc),
 * then phi in [0, 2 pi); frame b1 = normalize(h x a), b2 = a x b1, h = x
 * unless |a.x| >= 0.9, then y. */
static V3 spot_dir(rng_t *rg, V3 a, double cc) {
    double u = gen_range(rg, 0.0, 1.0);
    double phi = gen_range(rg, 0.0, 2.0 * PI_D);
    double c = 1.0 - u * (1.0 - cc);
    double s = sqrt(1.0 - c * c);
    double sn = m_sin(phi), cs = m_cos(phi);
    V3 h = fabs(a.x) < 0.9 ? v3(1.0, 0.0, 0.0) : v3(0.0, 1.0, 0.0);
    V3 b1 = v3(1.0, 0.0, 0.0);
    vnormalize(vcross(h, a), &b1);
    V3 b2 = vcross(a, b1);
    V3 d = a;
    vnormalize(vadd(vadd(vmul(b1, s * cs), vmul(b2, s * sn)), vmul(a, c)), &d);
    return d;
}

/* Light::generate_photon, light.rs:67-91; select_wavelength, light.rs:157-160 */
static photon_t generate_photon(const orc_light *l, rng_t *rg) {
    photon_t ph;
    ph.wl = orc_decide_wavelength(l->color, gen_range(rg, 0.0, 1.0));
    if (l->kind == ORC_LPOINT) {
        ph.pos = v3p(l->pos);
        ph.dir = random_dir(rg);
    } else if (l->kind == ORC_LSPOT) {
        ph.pos = v3p(l->pos);
        ph.dir = spot_dir(rg, v3p(l->dir), l->dir1[0]);
    } else if (l->kind == ORC_LPARALLELOGRAM) {
        double t1 = gen_range(rg, 0.0, 1.0);
        double t2 = gen_range(rg, 0.0, 1.0);
        V3 d = diffuse_reflection(rg, v3p(l->nvec));
        ph.pos = vadd(vadd(v3p(l->pos), smul(t1, v3p(l->dir1))), smul(t2, v3p(l->dir2)));
        ph.dir = d;
    } else {
        double t1 = gen_range(rg, 0.0, 1.0);
        double t2 = gen_range(rg, 0.0, 1.0);
        ph.pos = vadd(vadd(v3p(l->pos), smul(t1, v3p(l->dir1))), smul(t2, v3p(l->dir2)));
        ph.dir = v3p(l->dir);
    }
    return ph;
}

typedef struct { int wl; V3 pos, dir; int level; } stored_t;

/* trace_photon, tracer.rs:31-81 with reflect_diff/spec/trans :83-125 and
 * Surface::next_direction surface.rs:211-258, unrolled over levels.  The
 * reference recurses once per level (no branching), so a loop is exact. */
static int trace_photon(const orc_scene *sc, int uc, uint64_t seed, uint32_t pass,
                        uint32_t item, photon_t ph, stored_t *out) {
    int m0 = -1, nst = 0;
    for (int l = 0; l < MAX_TRACE; l++) {
        isect_t is;
        if (!intersect(sc, ph.pos, ph.dir, &is)) break;
        const orc_material *mate = &sc->mats[sc->objs[is.obj].material];
        rng_t rg;
        rng_init(&rg, seed, item, pass, TAG_BOUNCE | (uint32_t)l);
        int cont = 0, nmed = m0;
        V3 nd = v3(0, 0, 0);
        if (mate->surface == ORC_SIMPLE) {
            if (rr1(&rg, sf_roughness(mate)) == 0) {                 /* reflect_diff */
                if (rr1(&rg, sf_albedo_diff(mate, ph.wl)) == 0) {
                    nd = diffuse_reflection(&rg, is.n);
                    cont = 1;
                }
            } else {                                                  /* reflect_spec */
                double cos1;
                V3 rdir = specular_reflection(is.n, ph.dir, &cos1);
                double f = orc_schlick(sf_albedo_spec(mate, ph.wl), cos1);
                if (rr1(&rg, f) == 0) {
                    nd = rdir; cont = 1;
                } else if (mate->ior[ph.wl] == 0.0) {
                    /* absorbed */
                } else {                                              /* reflect_trans */
                    double eta = orc_relative_ior(mat_of(sc, m0)->ior[ph.wl], mate->ior[ph.wl]);
                    double c2;
                    V3 td;
                    if (specular_refraction(is.n, ph.dir, eta, &td, &c2)) {
                        nmed = vdot(td, is.n) < 0.0 ? sc->objs[is.obj].material : -1;
                        nd = td; cont = 1;
                    }
                }
            }
        } else if (mate->surface == ORC_TS) {
            double eta = orc_relative_ior(mat_of(sc, m0)->ior[ph.wl], mate->ior[ph.wl]);
            double cos1, cos2;
            V3 rdir0 = specular_reflection(is.n, ph.dir, &cos1);
            V3 rdir = reflection_glossy(&rg, is.n, rdir0, sf_power_glossy(mate));
            V3 hvec, td;
            if (!vnormalize(vsub(rdir, ph.dir), &hvec)) hvec = is.n;
            int has_t = specular_refraction(hvec, ph.dir, eta, &td, &cos2);
            double cos = cos1 < cos2 ? cos1 : cos2;
            double f = orc_schlick(sf_albedo_spec(mate, ph.wl), cos);
            if (rr1(&rg, f) == 0) {
                nd = rdir; cont = 1;                                  /* reflect: keep m0 */
            } else if (rr1(&rg, sf_albedo_diff(mate, ph.wl)) == 1) {
                /* absorbed */
            } else if (rr1(&rg, mate->scatter) == 0) {
                nd = diffuse_reflection(&rg, is.n); cont = 1;
            } else if (has_t) {
                nd = td; cont = 1; nmed = sc->objs[is.obj].material;  /* tracer.rs:68 */
            }
        }
        if ((!uc || l > 0) && sf_store(mate)) {
            out[nst].wl = ph.wl; out[nst].pos = is.pos; out[nst].dir = ph.dir; out[nst].level = l;
            nst++;
        }
        if (!cont) break;
        ph.pos = is.pos; ph.dir = nd; m0 = nmed;
    }
    return nst;
}

int64_t orc_trace_photons(const orc_scene *sc, int64_t nphoton, int uc, uint64_t seed,
                          uint32_t pass, double *pos, double *dir, uint8_t *wl,
                          int32_t *emit_idx, int8_t *level, int64_t cap,
                          double *power_out, int64_t *n_emitted_out) {
    /* ppmpa.rs:30-31, :70-72 */
    double total = 0.0;
    for (int i = 0; i < sc->n_lights; i++) total = total + sc->lights[i].flux;
    double power = total / (double)nphoton;
    int64_t ns[64], nem = 0;
    for (int i = 0; i < sc->n_lights && i < 64; i++) {
        ns[i] = (int64_t)llround(sc->lights[i].flux / power);
        nem += ns[i];
    }
    if (power_out) *power_out = power;
    if (n_emitted_out) *n_emitted_out = nem;
    stored_t *slots = (stored_t *)malloc(sizeof(stored_t) * (size_t)(nem > 0 ? nem : 1) * MAX_TRACE);
    int *cnt = (int *)calloc((size_t)(nem > 0 ? nem : 1), sizeof(int));
#pragma omp parallel for schedule(dynamic, 1024) num_threads(orc_get_threads())
    for (int64_t e = 0; e < nem; e++) {
        int li = 0;
        int64_t base = 0;
        while (li < sc->n_lights - 1 && e >= base + ns[li]) { base += ns[li]; li++; }
        rng_t rg;
        rng_init(&rg, seed, (uint32_t)e, pass, TAG_EMIT);
        photon_t ph = generate_photon(&sc->lights[li], &rg);
        cnt[e] = trace_photon(sc, uc, seed, pass, (uint32_t)e, ph, slots + e * MAX_TRACE);
    }
    int64_t total_st = 0;
    for (int64_t e = 0; e < nem; e++) total_st += cnt[e];
    if (total_st > cap) { free(slots); free(cnt); return -total_st; }
    int64_t k = 0;
    for (int64_t e = 0; e < nem; e++) {
        for (int j = cnt[e] - 1; j >= 0; j--) {   /* deepest first (tracer.rs:77-80) */
            const stored_t *s = &slots[e * MAX_TRACE + j];
            if (pos) { pos[3 * k] = s->pos.x; pos[3 * k + 1] = s->pos.y; pos[3 * k + 2] = s->pos.z; }
            if (dir) { dir[3 * k] = s->dir.x; dir[3 * k + 1] = s->dir.y; dir[3 * k + 2] = s->dir.z; }
            if (wl) wl[k] = (uint8_t)s->wl;
            if (emit_idx) emit_idx[k] = (int32_t)e;
            if (level) level[k] = (int8_t)s->level;
            k++;
        }
    }
    free(slots); free(cnt);
    return total_st;
}

/* ------------------------------------------------------------------------ */
/* In-radius query: restated kdtree 0.5.1 `within` semantics over a grid    */
/* ------------------------------------------------------------------------ */
typedef struct {
    double org[3], cell;
    int64_t dim[3];
    int64_t *start;     /* ncell + 1 */
    int32_t *idx;       /* photons sorted by cell, ascending index inside */
} grid_t;

static inline int64_t clampi(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

static void grid_build(grid_t *g, const double *pp, int64_t np, double cell) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < np; i++)
        for (int a = 0; a < 3; a++) {
            double v = pp[3 * i + a];
            if (v < lo[a]) lo[a] = v;
            if (v > hi[a]) hi[a] = v;
        }
    if (np == 0) { lo[0] = lo[1] = lo[2] = 0; hi[0] = hi[1] = hi[2] = 0; }
    if (!(cell > 0)) cell = 1.0;
    for (;;) {
        int64_t tot = 1;
        for (int a = 0; a < 3; a++) {
            g->dim[a] = (int64_t)floor((hi[a] - lo[a]) / cell) + 1;
            tot *= g->dim[a];
        }
        if (tot <= (int64_t)1 << 24) break;
        cell *= 1.5;
    }
    for (int a = 0; a < 3; a++) g->org[a] = lo[a];
    g->cell = cell;
    int64_t nc = g->dim[0] * g->dim[1] * g->dim[2];
    g->start = (int64_t *)calloc((size_t)nc + 1, sizeof(int64_t));
    g->idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(np > 0 ? np : 1));
    int64_t *key = (int64_t *)malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));
    for (int64_t i = 0; i < np; i++) {
        int64_t c[3];
        for (int a = 0; a < 3; a++)
            c[a] = clampi((int64_t)floor((pp[3 * i + a] - g->org[a]) / cell), 0, g->dim[a] - 1);
        key[i] = (c[2] * g->dim[1] + c[1]) * g->dim[0] + c[0];
        g->start[key[i] + 1]++;
    }
    for (int64_t c = 0; c < nc; c++) g->start[c + 1] += g->start[c];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
    memcpy(fill, g->start, sizeof(int64_t) * (size_t)nc);
    for (int64_t i = 0; i < np; i++) g->idx[fill[key[i]]++] = (int32_t)i;
    free(fill); free(key);
}

static void grid_free(grid_t *g) { free(g->start); free(g->idx); }

/* squared_euclidean(query, point) <= r2 (kdtree 0.5.1 within) */
static inline double sq_euclid(const double *q, const double *p) {
    double dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
    double s = 0.0;
    s = s + dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return s;
}

typedef struct { double d; int32_t i; } nb_t;

static int nb_cmp_idx(const void *a, const void *b) {
    int32_t x = ((const nb_t *)a)->i, y = ((const nb_t *)b)->i;
    return (x > y) - (x < y);
}
static int nb_cmp_dist(const void *a, const void *b) {
    const nb_t *x = (const nb_t *)a, *y = (const nb_t *)b;
    if (x->d < y->d) return -1;
    if (x->d > y->d) return 1;
    return (x->i > y->i) - (x->i < y->i);
}

/* collect neighbours of q within r2; returns count, (re)allocates *buf */
static int64_t grid_query(const grid_t *g, const double *pp, const double *q, double r2,
                          nb_t **buf, int64_t *bufcap) {
    double r = sqrt(r2);
    int64_t lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = clampi((int64_t)floor((q[a] - r - g->org[a]) / g->cell) - 1, 0, g->dim[a] - 1);
        hi[a] = clampi((int64_t)floor((q[a] + r - g->org[a]) / g->cell) + 1, 0, g->dim[a] - 1);
    }
    int64_t n = 0;
    for (int64_t z = lo[2]; z <= hi[2]; z++)
        for (int64_t y = lo[1]; y <= hi[1]; y++) {
            int64_t c0 = (z * g->dim[1] + y) * g->dim[0];
            for (int64_t k = g->start[c0 + lo[0]]; k < g->start[c0 + hi[0] + 1]; k++) {
                int32_t i = g->idx[k];
                double d = sq_euclid(q, pp + 3 * (int64_t)i);
                if (d <= r2) {
                    if (n == *bufcap) {
                        *bufcap = *bufcap ? *bufcap * 2 : 256;
                        *buf = (nb_t *)realloc(*buf, sizeof(nb_t) * (size_t)*bufcap);
                    }
                    (*buf)[n].d = d; (*buf)[n].i = i; n++;
                }
            }
        }
    return n;
}

int64_t orc_within(const double *ppos, int64_t np, const double *q, int64_t nq,
                   const double *r2, int64_t *offsets, int32_t *idx, int64_t cap) {
    double rmax = 0.0;
    for (int64_t i = 0; i < nq; i++) if (r2[i] > rmax) rmax = r2[i];
    rmax = sqrt(rmax);
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < np; i++)
        for (int a = 0; a < 3; a++) {
            if (ppos[3 * i + a] < lo[a]) lo[a] = ppos[3 * i + a];
            if (ppos[3 * i + a] > hi[a]) hi[a] = ppos[3 * i + a];
        }
    double vol = 1.0;
    for (int a = 0; a < 3; a++) vol *= (np > 0 ? (hi[a] - lo[a]) : 0.0) + 1e-9;
    double cell = np > 0 ? cbrt(vol * 4.0 / (double)np) : 1.0;
    if (rmax > 0 && cell > rmax) cell = rmax;
    grid_t g;
    grid_build(&g, ppos, np, cell);
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nq > 0 ? nq : 1));
#pragma omp parallel num_threads(orc_get_threads())
    {
        nb_t *buf = NULL;
        int64_t bc = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < nq; i++) cnt[i] = grid_query(&g, ppos, q + 3 * i, r2[i], &buf, &bc);
        free(buf);
    }
    int64_t total = 0;
    for (int64_t i = 0; i < nq; i++) {
        if (offsets) offsets[i] = total;
        total += cnt[i];
    }
    if (offsets) offsets[nq] = total;
    if (idx && offsets && total <= cap) {
#pragma omp parallel num_threads(orc_get_threads())
        {
            nb_t *buf = NULL;
            int64_t bc = 0;
#pragma omp for schedule(dynamic, 64)
            for (int64_t i = 0; i < nq; i++) {
                int64_t n = grid_query(&g, ppos, q + 3 * i, r2[i], &buf, &bc);
                qsort(buf, (size_t)n, sizeof(nb_t), nb_cmp_idx);
                for (int64_t k = 0; k < n; k++) idx[offsets[i] + k] = buf[k].i;
            }
            free(buf);
        }
    }
    free(cnt);
    grid_free(&g);
    return total;
}

/* filters, tracer.rs:197-216 */
double orc_filter_cone(double d, double rmax) {
    double d2 = sqrt(d / rmax) / K_CONE;
    return d2 > 1.0 ? 0.0 : (1.0 - d2) / FAC_K;
}
double orc_filter_gauss_corr(double d, double rmax, double corr) {
    double e_r = 1.0 - m_exp(-G_BETA * d / (rmax * 2.0));
    return e_r > G_E_BETA ? 0.0 : G_ALPHA * (1.0 - e_r / G_E_BETA) + corr;
}
double orc_filter_gauss(double d, double rmax) { return orc_filter_gauss_corr(d, rmax, G_CORR); }

typedef struct {
    const double *pos, *dir;
    const uint8_t *wl;
    int64_t np;
    double pw, r2;
    int pfilter;
    grid_t g;
} pmap_t;

/* estimate_radiance, tracer.rs:179-195 */
static V3 estimate_radiance(const pmap_t *pm, V3 p, V3 n, nb_t **buf, int64_t *bc) {
    double q[3] = {p.x, p.y, p.z};
    int64_t k = grid_query(&pm->g, pm->pos, q, pm->r2, buf, bc);
    if (k == 0) return v3(0, 0, 0);
    qsort(*buf, (size_t)k, sizeof(nb_t), nb_cmp_dist);
    V3 rad = v3(0, 0, 0);
    for (int64_t j = 0; j < k; j++) {
        double d = (*buf)[j].d;
        int32_t i = (*buf)[j].i;
        double wt = 1.0;
        if (pm->pfilter == ORC_PF_CONE) wt = orc_filter_cone(d, pm->r2);
        else if (pm->pfilter == ORC_PF_GAUSS) wt = orc_filter_gauss(d, pm->r2);
        double pw = wt * pm->pw;
        double cos0 = vdot(n, v3p(pm->dir + 3 * (int64_t)i));   /* optics.rs:224-236 */
        double pw2 = cos0 < 0.0 ? pw * -cos0 : 0.0;
        V3 c = v3(0, 0, 0);
        if (pm->wl[i] == 0) c.x = pw2; else if (pm->wl[i] == 1) c.y = pw2; else c.z = pw2;
        rad = vadd(rad, c);
    }
    return vmul(rad, ONE_PI / pm->r2);
}

void orc_estimate(const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                  const double *qpos, const double *qnrm, int64_t nq,
                  double r2, double pw, int pfilter, double *rgb) {
    pmap_t pm = {ppos, pdir, pwl, np, pw, r2, pfilter, {{0}, 0, {0}, NULL, NULL}};
    grid_build(&pm.g, ppos, np, sqrt(r2));
#pragma omp parallel num_threads(orc_get_threads())
    {
        nb_t *buf = NULL;
        int64_t bc = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < nq; i++) {
            V3 r = estimate_radiance(&pm, v3p(qpos + 3 * i), v3p(qnrm + 3 * i), &buf, &bc);
            rgb[3 * i] = r.x; rgb[3 * i + 1] = r.y; rgb[3 * i + 2] = r.z;
        }
        free(buf);
    }
    grid_free(&pm.g);
}

static double g_last_query_seconds = 0.0;
double orc_last_query_seconds(void) { return g_last_query_seconds; }

static double wall_seconds(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

void orc_estimate_radii(const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                        const double *qpos, const double *qnrm, int64_t nq,
                        const double *r2, double pw, int pfilter, double *rgb) {
    double rmax2 = 0.0;
    for (int64_t i = 0; i < nq; i++) if (r2[i] > rmax2) rmax2 = r2[i];
    pmap_t pm = {ppos, pdir, pwl, np, pw, rmax2, pfilter, {{0}, 0, {0}, NULL, NULL}};
    grid_build(&pm.g, ppos, np, sqrt(rmax2));
    double t0 = wall_seconds();
#pragma omp parallel num_threads(orc_get_threads())
    {
        nb_t *buf = NULL;
        int64_t bc = 0;
        pmap_t qm = pm;
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < nq; i++) {
            qm.r2 = r2[i];
            V3 r = estimate_radiance(&qm, v3p(qpos + 3 * i), v3p(qnrm + 3 * i), &buf, &bc);
            rgb[3 * i] = r.x; rgb[3 * i + 1] = r.y; rgb[3 * i + 2] = r.z;
        }
        free(buf);
    }
    g_last_query_seconds = wall_seconds() - t0;
    grid_free(&pm.g);
}

/* SplitMix64's output function (Steele, Lea and Flood, OOPSLA 2014) of
 * (slot + 1) times its increment: the per-slot term of a neighbour-set
 * checksum (the same function as the GPU export's). */
static uint64_t slot_mix(uint64_t slot) {
    uint64_t z = (slot + 1u) * 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

/* The flux sums of estimate_radiance (tracer.rs:179-195) before its pw and
 * 1/(pi r2) factors, per query: for the photons within r2 (kdtree within,
 * tracer.rs:180), in the reference's ascending-distance order, sums[3i+wl]
 * += wt(d, r2) * max(0, -n . dir) (filters tracer.rs:197-216,
 * photon_to_radiance optics.rs:224-236); count[i] = number in radius;
 * hash[i] = sum of slot_mix(photon index) mod 2^64. */
void orc_gather_sums(const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                     const double *qpos, const double *qnrm, int64_t nq, double r2, int pfilter,
                     int64_t *count, uint64_t *hash, double *sums) {
    grid_t g;
    grid_build(&g, ppos, np, sqrt(r2));
#pragma omp parallel num_threads(orc_get_threads())
    {
        nb_t *buf = NULL;
        int64_t bc = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < nq; i++) {
            int64_t k = grid_query(&g, ppos, qpos + 3 * i, r2, &buf, &bc);
            qsort(buf, (size_t)k, sizeof(nb_t), nb_cmp_dist);
            V3 n = v3p(qnrm + 3 * i);
            double s[3] = {0.0, 0.0, 0.0};
            uint64_t h = 0;
            for (int64_t j = 0; j < k; j++) {
                double d = buf[j].d;
                int32_t p = buf[j].i;
                double wt = 1.0;
                if (pfilter == ORC_PF_CONE) wt = orc_filter_cone(d, r2);
                else if (pfilter == ORC_PF_GAUSS) wt = orc_filter_gauss(d, r2);
                double cos0 = vdot(n, v3p(pdir + 3 * (int64_t)p));
                double w = cos0 < 0.0 ? wt * -cos0 : 0.0;
                s[pwl[p] < 2 ? pwl[p] : 2] += w;
                h += slot_mix((uint64_t)p);
            }
            count[i] = k;
            hash[i] = h;
            for (int c = 0; c < 3; c++) sums[3 * i + c] = s[c];
        }
        free(buf);
    }
    grid_free(&g);
}

/* ------------------------------------------------------------------------ */
/* Direct light: get_radiance_from_light / illuminated, tracer.rs:263-290;  */
/* Light::get_direction / get_radiance, light.rs:93-150.  The reference     */
/* zips get_radiance(dists) -- which starts with an extra RADIANCE0 -- with */
/* coss, so sample k's cos multiplies sample k-1's radiance and the first   */
/* cos multiplies zero.  Restated as is.                                    */
/* ------------------------------------------------------------------------ */
static const double TSS[5] = {0.1, 0.3, 0.5, 0.7, 0.9};

static V3 light_radiance(const orc_light *l, double d) {
    double l0;
    if (l->kind == ORC_LPOINT || l->kind == ORC_LSPOT) l0 = l->flux / (PI4_D * d);
    else if (l->kind == ORC_LPARALLELOGRAM) l0 = (2.0 * l->flux * PARA_DIV * PARA_DIV) / (PI4_D * d);
    else l0 = l->flux;
    return v3(l->color[0] * l0, l->color[1] * l0, l->color[2] * l0);
}

static V3 radiance_from_light(const orc_scene *sc, V3 p, V3 n, const orc_light *l) {
    V3 lds[25];
    int nl = 0;
    if (l->kind == ORC_LPOINT || l->kind == ORC_LSPOT) {
        lds[nl++] = vsub(v3p(l->pos), p);
    } else if (l->kind == ORC_LPARALLELOGRAM) {
        for (int a = 0; a < 5; a++)
            for (int b = 0; b < 5; b++) {
                V3 sp = vadd(vadd(v3p(l->pos), smul(TSS[a], v3p(l->dir1))), smul(TSS[b], v3p(l->dir2)));
                V3 d = vsub(sp, p);
                if (vdot(v3p(l->nvec), d) < 0.0) lds[nl++] = d;
            }
    } else {
        V3 d = vsub(v3p(l->pos), p);
        double cos0 = vdot(v3p(l->nvec), d);
        if (!(cos0 > 0.0)) {
            V3 dt2 = vneg(v3p(l->dir));
            double t;
            if (method_moller(2.0, v3p(l->pos), v3p(l->dir1), v3p(l->dir2), p, dt2, &t))
                lds[nl++] = smul(t, dt2);
        }
    }
    double dists[25], coss[25];
    int k = 0;
    for (int i = 0; i < nl; i++) {
        V3 ld3;
        if (!vnormalize(lds[i], &ld3)) continue;
        double cos0 = vdot(n, ld3);
        if (cos0 < 0.0) continue;
        isect_t is;
        if (!intersect(sc, p, ld3, &is)) continue;
        double sq_ldist = vdot(lds[i], lds[i]);
        V3 dd = vsub(is.pos, p);
        double sq_odist = vdot(dd, dd);
        if (sq_ldist - sq_odist > 0.002) continue;
        dists[k] = sq_ldist; coss[k] = cos0 * cos0; k++;
    }
    V3 rad = v3(0, 0, 0);
    for (int i = 0; i < k; i++) {
        V3 r = i == 0 ? v3(0, 0, 0) : light_radiance(l, dists[i - 1]);
        rad = vadd(rad, vmul(r, coss[i]));
    }
    return rad;
}

/* ------------------------------------------------------------------------ */
/* Eye path: trace_ray, tracer.rs:129-177 (literal recursion)               */
/* ------------------------------------------------------------------------ */
typedef struct {
    const orc_scene *sc;
    const pmap_t *pm;
    int uc;
    uint64_t seed;
    uint32_t pass, pixel;
    nb_t **buf;
    int64_t *bc;
} eye_ctx;

static V3 trace_ray(const eye_ctx *ec, int m0, int l, uint32_t node, V3 rp, V3 rd) {
    if (l >= MAX_TRACE) return v3(0, 0, 0);
    isect_t is;
    if (!intersect(ec->sc, rp, rd, &is)) return v3(0, 0, 0);
    const orc_scene *sc = ec->sc;
    int mid = sc->objs[is.obj].material;
    const orc_material *mate = &sc->mats[mid];
    V3 di = v3(0, 0, 0);
    if (ec->uc)
        for (int i = 0; i < sc->n_lights; i++)
            di = vadd(di, radiance_from_light(sc, is.pos, is.n, &sc->lights[i]));
    di = vadd(di, estimate_radiance(ec->pm, is.pos, is.n, ec->buf, ec->bc));
    double cos1, cos2;
    V3 rdir0 = specular_reflection(is.n, rd, &cos1);
    rng_t rg;
    rng_init(&rg, ec->seed, ec->pixel, ec->pass, TAG_EYE | node);
    V3 rdir = reflection_glossy(&rg, is.n, rdir0, sf_power_glossy(mate));
    V3 si = v3(0, 0, 0);
    if (sf_reflect(mate, cos1)) si = trace_ray(ec, m0, l + 1, 2 * node, is.pos, rdir);
    double eta = relative_ior_average(mat_of(sc, m0)->ior, mate->ior);
    V3 hvec, td;
    if (!vnormalize(vsub(rdir, rd), &hvec)) hvec = is.n;
    int has_t = specular_refraction(hvec, rd, eta, &td, &cos2);
    V3 ti = v3(0, 0, 0);
    if (has_t && sf_refract(mate, cos1))
        ti = trace_ray(ec, is.in ? mid : -1, l + 1, 2 * node + 1, is.pos, td);
    double cos = cos1 < cos2 ? cos1 : cos2;
    V3 em = vmul(v3p(mate->emittance), SR_HALF);
    return vadd(em, sf_bsdf(mate, cos, di, si, ti));
}

/* Camera::generate_ray, camera.rs:58-75 */
static void generate_ray(const orc_camera *c, rng_t *rg, double y, double x, V3 *rp, V3 *rd) {
    V3 blur = v3(0, 0, 0);
    if (c->blur) {
        double r1 = gen_range(rg, -0.5, 0.5);
        double r2 = gen_range(rg, -0.5, 0.5);
        blur = vadd(smul(r1, v3p(c->eex)), smul(r2, v3p(c->eey)));
    }
    double r3 = 0.0, r4 = 0.0;
    if (c->progressive && c->antialias) {
        r3 = gen_range(rg, -0.5, 0.5);
        r4 = gen_range(rg, -0.5, 0.5);
    }
    *rp = vadd(v3p(c->eye_pos), blur);
    V3 ed = vsub(vadd(vadd(v3p(c->origin), smul(x + r3, v3p(c->esx))), smul(y + r4, v3p(c->esy))), blur);
    vnormalize(ed, rd);
}

/* read_camera derived values, camera.rs:150-175 */
void orc_camera_derive(orc_camera *c) {
    const double SENSOR = 35.0 / 1000.0, ISO = 100.0, FNUM = 4.9, SHUT = 1.0 / 250.0;
    V3 eye = v3p(c->eye_pos), tgt = v3p(c->target), up = v3p(c->upper);
    V3 ez = {0, 0, 0}, ex = ez, ey = ez;
    vnormalize(vsub(tgt, eye), &ez);
    vnormalize(vcross(up, ez), &ex);
    vnormalize(vcross(ex, ez), &ey);
    double step = (c->focus * SENSOR / c->focal_len) / (double)c->xreso;
    V3 esx = smul(step, ex), esy = smul(step, ey);
    double ea = c->focal_len / c->f_number;
    V3 eex = smul(ea, ex), eey = smul(ea, ey);
    double lx = (double)(c->xreso / 2), ly = (double)(c->yreso / 2);
    V3 orig = vsub(vsub(smul(c->focus, ez), smul(lx - 0.5, esx)), smul(ly - 0.5, esy));
    c->photon_power = c->blur ? c->iso_sens / ISO * FNUM / c->f_number * c->shut_speed / SHUT : 1.0;
    V3 edir;
    vnormalize(vsub(tgt, eye), &edir);
    double *dst[6] = {c->eye_dir, c->origin, c->esx, c->esy, c->eex, c->eey};
    V3 src[6] = {edir, orig, esx, esy, eex, eey};
    for (int i = 0; i < 6; i++) { dst[i][0] = src[i].x; dst[i][1] = src[i].y; dst[i][2] = src[i].z; }
}

/* trace_ray_classic, tracer.rs:221-259 (Whitted-style: no photon map).
 * di = direct light of every light (always) + the camera's ambient; the
 * reflected child follows the exact mirror direction; refraction bends about
 * the surface normal and the child's medium is the hit material when the
 * refracted ray goes into the surface (tdir . n < 0), air otherwise; the
 * bsdf takes cos1. */
static V3 trace_ray_classic(const orc_scene *sc, const orc_camera *cam, int m0, int l, V3 rp, V3 rd) {
    if (l >= MAX_TRACE) return v3(0, 0, 0);
    isect_t is;
    if (!intersect(sc, rp, rd, &is)) return v3(0, 0, 0);
    int mid = sc->objs[is.obj].material;
    const orc_material *mate = &sc->mats[mid];
    double cos1, cos2;
    V3 rdir = specular_reflection(is.n, rd, &cos1);
    V3 di = v3(0, 0, 0);
    for (int i = 0; i < sc->n_lights; i++) di = vadd(di, radiance_from_light(sc, is.pos, is.n, &sc->lights[i]));
    di = vadd(di, v3p(cam->ambient));
    V3 si = v3(0, 0, 0);
    if (sf_reflect(mate, cos1)) si = trace_ray_classic(sc, cam, m0, l + 1, is.pos, rdir);
    double eta = relative_ior_average(mat_of(sc, m0)->ior, mate->ior);
    V3 td;
    int has_t = specular_refraction(is.n, rd, eta, &td, &cos2);
    V3 ti = v3(0, 0, 0);
    if (has_t && sf_refract(mate, cos1))
        ti = trace_ray_classic(sc, cam, vdot(td, is.n) < 0.0 ? mid : -1, l + 1, is.pos, td);
    V3 em = vmul(v3p(mate->emittance), SR_HALF);
    return vadd(em, sf_bsdf(mate, cos1, di, si, ti));
}

void orc_classic_pass(const orc_scene *sc, const orc_camera *cam, uint64_t seed, uint32_t pass, double *image) {
    int64_t npx = (int64_t)cam->xreso * cam->yreso;
#pragma omp parallel for schedule(dynamic, 64) num_threads(orc_get_threads())
    for (int64_t p = 0; p < npx; p++) {
        int64_t y = p / cam->xreso, x = p % cam->xreso;
        rng_t rg;
        rng_init(&rg, seed, (uint32_t)p, pass, TAG_CAMERA);
        V3 rp, rd;
        generate_ray(cam, &rg, (double)y, (double)x, &rp, &rd);
        V3 r = trace_ray_classic(sc, cam, -1, 0, rp, rd);
        image[3 * p] += r.x; image[3 * p + 1] += r.y; image[3 * p + 2] += r.z;
    }
}

void orc_eye_pass(const orc_scene *sc, const orc_camera *cam,
                  const double *ppos, const double *pdir, const uint8_t *pwl, int64_t np,
                  double r2, double pw, int uc, uint64_t seed, uint32_t pass, double *image) {
    pmap_t pm = {ppos, pdir, pwl, np, pw, r2, cam->pfilter, {{0}, 0, {0}, NULL, NULL}};
    grid_build(&pm.g, ppos, np, sqrt(r2));
    int64_t npx = (int64_t)cam->xreso * cam->yreso;
#pragma omp parallel num_threads(orc_get_threads())
    {
        nb_t *buf = NULL;
        int64_t bc = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t p = 0; p < npx; p++) {
            int64_t y = p / cam->xreso, x = p % cam->xreso;
            rng_t rg;
            rng_init(&rg, seed, (uint32_t)p, pass, TAG_CAMERA);
            V3 rp, rd;
            generate_ray(cam, &rg, (double)y, (double)x, &rp, &rd);
            eye_ctx ec = {sc, &pm, uc, seed, pass, (uint32_t)p, &buf, &bc};
            V3 r = trace_ray(&ec, -1, 0, 1u, rp, rd);
            image[3 * p] += r.x; image[3 * p + 1] += r.y; image[3 * p + 2] += r.z;
        }
        free(buf);
    }
    grid_free(&pm.g);
}

/* PA radius schedule: util/iterator.rb:33-38 (offset 1), util/radius.rb:13-17 (offset 0) */
void orc_radius_schedule(double r0, double alpha, int off, int passes, double *r2) {
    double r = r0 * r0;
    for (int k = 0; k < passes; k++) {
        r2[k] = r;
        double i = (double)(k + off);
        r = r * ((i + alpha) / (i + 1.0));
    }
}

void orc_render(const orc_scene *sc, const orc_camera *cam, int64_t nphoton, int passes,
                double r0, double alpha, int off, int uc, uint64_t seed, double *image) {
    int64_t npx = (int64_t)cam->xreso * cam->yreso;
    double *r2 = (double *)malloc(sizeof(double) * (size_t)(passes > 0 ? passes : 1));
    orc_radius_schedule(r0, alpha, off, passes, r2);
    memset(image, 0, sizeof(double) * 3 * (size_t)npx);
    int64_t cap = nphoton * MAX_TRACE + 64;
    double *pos = (double *)malloc(sizeof(double) * 3 * (size_t)cap);
    double *dir = (double *)malloc(sizeof(double) * 3 * (size_t)cap);
    uint8_t *wl = (uint8_t *)malloc((size_t)cap);
    for (int k = 0; k < passes; k++) {
        double pw;
        int64_t nem;
        int64_t n = orc_trace_photons(sc, nphoton, uc, seed, (uint32_t)k, pos, dir, wl, NULL, NULL, cap, &pw, &nem);
        if (n < 0) n = 0;
        orc_eye_pass(sc, cam, pos, dir, wl, n, r2[k], pw, uc, seed, (uint32_t)k, image);
    }
    for (int64_t i = 0; i < 3 * npx; i++) image[i] = image[i] / (double)passes;
    free(pos); free(dir); free(wl); free(r2);
}
