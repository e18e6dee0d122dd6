// ppm_common.cuh -- device building blocks shared by the FP64 (plain) and
// FP32 (mixed) paths: 3-vectors, the Philox4x32-10 stream, FP64 elementary
// functions and the device-side scene tables.
//
// The FP64 instantiations are compiled with --fmad=false so every double
// expression rounds exactly as written; the operation order follows the
// reference's Rust expressions (src/ray/algebra.rs, physics.rs), which makes
// the FP64 photon paths reproducible bit for bit on the host.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ppm {

constexpr int MAX_TRACE = 10;                    // src/tracer.rs:27
constexpr double NEARLY0 = 0.0001;               // src/ray/mod.rs:16
constexpr double PI_D = 0x1.921fb54442d18p+1;
constexpr double PI4_D = PI_D * 4.0;             // src/ray/mod.rs:18
constexpr double ONE_PI_D = 1.0 / PI_D;          // src/tracer.rs:24
constexpr double SR_HALF_D = 1.0 / (2.0 * PI_D); // src/tracer.rs:25
constexpr double PARA_DIV = 0.2;                 // src/ray/light.rs:162

// random-stream tags (counter word 2)
constexpr uint32_t TAG_EMIT = 0x01000000u;
constexpr uint32_t TAG_BOUNCE = 0x02000000u;
constexpr uint32_t TAG_CAMERA = 0x03000000u;
constexpr uint32_t TAG_EYE = 0x04000000u;

enum { SH_POINT = 0, SH_PLAIN = 1, SH_SPHERE = 2, SH_POLYGON = 3, SH_PARALLELOGRAM = 4 };
enum { SF_NOTHING = 0, SF_SIMPLE = 1, SF_TS = 2 };
enum { LT_POINT = 0, LT_PARALLELOGRAM = 1, LT_SUN = 2, LT_SPOT = 3 };
enum { PF_NONE = 0, PF_CONE = 1, PF_GAUSS = 2 };

// ---------------------------------------------------------------------------
// 3-vectors.  Operator order mirrors src/ray/algebra.rs:146-180.
// ---------------------------------------------------------------------------
template <typename T>
struct V3 {
    T x, y, z;
};

template <typename T> __host__ __device__ __forceinline__ V3<T> mk3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> ld3(const T *p) { return V3<T>{p[0], p[1], p[2]}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> hmul(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename T> __host__ __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> __host__ __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <typename T> __host__ __device__ __forceinline__ bool any_nz(V3<T> a) { return a.x != T(0) || a.y != T(0) || a.z != T(0); }

__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }

// Vector3::normalize (algebra.rs:186-194): multiply by the reciprocal norm.
template <typename T>
__device__ __forceinline__ bool normalize(V3<T> a, V3<T> &out) {
    T n = dsqrt(dot(a, a));
    if (n == T(0)) return false;
    out = a * (T(1) / n);
    return true;
}

// ---------------------------------------------------------------------------
// Philox4x32-R (Salmon et al., SC'11).  key = seed, ctr = {item, pass, tag, block}.
// R = 10 for the FP64 path (the oracle's generator, bit for bit); R = 7 for
// the FP32 path, which is compared statistically: Salmon et al. report that
// Philox4x32 passes TestU01's BigCrush from 7 rounds on (10 is their margin),
// and 7 rounds take 4 % off the FP32 photon trace.
// ---------------------------------------------------------------------------
template <int R>
__host__ __device__ __forceinline__ void philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                                   uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int i = 0; i < R; i++) {
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

template <typename T> struct PhiloxRounds { static constexpr int value = 10; };
template <> struct PhiloxRounds<float> { static constexpr int value = 7; };

// Sequential draws of one event.  FP64: 52-bit uniforms (rand 0.6 float
// construction: (u64 >> 12) * 2^-52) from Philox4x32-10; FP32: 24-bit
// uniforms from Philox4x32-7.  An Rng instance serves one precision, named
// at init.  The first Philox block is computed by init, where the lanes of
// a warp are still together: an event's draws are taken in branches that
// differ per lane (diffuse, specular, glass), and a lazily computed first
// block would be computed once per branch a warp runs.
struct Rng {
    uint32_t k0, k1, item, pass, tag;
    uint32_t buf[4];
    int k;
    template <typename T>
    __device__ __forceinline__ void init(uint64_t seed, uint32_t it, uint32_t ps, uint32_t tg) {
        k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
        item = it; pass = ps; tag = tg; k = 0;
        philox4x32<PhiloxRounds<T>::value>(item, pass, tag, 0u, k0, k1, buf);
    }
    __device__ __forceinline__ uint64_t next64() {
        int w = k & 1;
        if (w == 0 && k > 0) philox4x32<10>(item, pass, tag, (uint32_t)(k >> 1), k0, k1, buf);
        uint64_t v = w ? ((uint64_t)buf[2] | ((uint64_t)buf[3] << 32)) : ((uint64_t)buf[0] | ((uint64_t)buf[1] << 32));
        k++;
        return v;
    }
    __device__ __forceinline__ double u64d() { return (double)(next64() >> 12) * 0x1p-52; }
    // FP32 draws use every 32-bit word of a block (4 draws per Philox call)
    __device__ __forceinline__ float u32f() {
        int w = k & 3;
        if (w == 0 && k > 0) philox4x32<7>(item, pass, tag, (uint32_t)(k >> 2), k0, k1, buf);
        uint32_t v = w == 0 ? buf[0] : (w == 1 ? buf[1] : (w == 2 ? buf[2] : buf[3]));
        k++;
        return (float)(v >> 8) * 0x1p-24f;
    }
};

template <typename T> struct RngT;
template <> struct RngT<double> {
    __device__ static __forceinline__ double u(Rng &r) { return r.u64d(); }
};
template <> struct RngT<float> {
    __device__ static __forceinline__ float u(Rng &r) { return r.u32f(); }
};

// rand 0.6 gen_range(lo, hi) = value0_1 * (hi - lo) + lo
template <typename T>
__device__ __forceinline__ T gen_range(Rng &r, T lo, T hi) { return RngT<T>::u(r) * (hi - lo) + lo; }

// ---------------------------------------------------------------------------
// FP64 elementary functions (identical operation sequences to the host
// oracle): sin/cos by Cody-Waite reduction with three 33-bit chunks of pi/2
// and Taylor polynomials on |r| <= pi/4; exp by ln2 reduction and a degree-14
// Taylor polynomial; log by 2*atanh((m-1)/(m+1)) with m in [sqrt(1/2), sqrt(2)].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pm_sincos(double x, double &s, double &c) {
    const double PIO2_1 = 0x1.921fb54400000p+0, PIO2_2 = 0x1.0b4611a600000p-34, PIO2_3 = 0x1.3198a2e037073p-69;
    double fk = floor(x * 0x1.45f306dc9c883p-1 + 0.5);
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
    int q = (int)(((long long)fk) & 3);
    if (q == 0) { s = sr; c = cr; }
    else if (q == 1) { s = cr; c = -sr; }
    else if (q == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
}

__device__ __forceinline__ double pm_scale2(double p, int k) {
    if (k > 1023) { p = p * __longlong_as_double((long long)(1023 + 1023) << 52); k -= 1023; }
    if (k < -1022) { p = p * __longlong_as_double((long long)(-1000 + 1023) << 52); k += 1000; }
    if (k < -1022) { p = p * __longlong_as_double((long long)(-1000 + 1023) << 52); k += 1000; }
    return p * __longlong_as_double((long long)(k + 1023) << 52);
}

__device__ __forceinline__ double pm_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000LL);
    if (x < -745.1332191019412) return 0.0;
    const double LN2_HI = 0x1.62e42fefa2000p-1, LN2_LO = 0x1.9ef35793c7673p-41;
    double fk = floor(x * 0x1.71547652b82fep+0 + 0.5);
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

__device__ __forceinline__ double pm_log(double x) {
    if (x != x || x < 0.0) return __longlong_as_double(0x7ff8000000000000LL);
    if (x == 0.0) return __longlong_as_double((long long)0xfff0000000000000ULL);
    if (__double_as_longlong(x) == 0x7ff0000000000000LL) return x;
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) {
        x = x * 0x1p54;
        b = (unsigned long long)__double_as_longlong(x);
        e = (int)((b >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    double m = __longlong_as_double((long long)((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL));
    if (m > 0x1.6a09e667f3bcdp+0) { m = m * 0.5; e += 1; }
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
    return (fe * 0x1.9ef35793c7673p-41 + lm) + fe * 0x1.62e42fefa2000p-1;
}

// Precision-dispatched elementary functions.  FP64: the functions above.
// FP32: CUDA's single-precision functions.
struct MathD {
    __device__ static __forceinline__ void sincos_(double x, double &s, double &c) { pm_sincos(x, s, c); }
    __device__ static __forceinline__ double pow_(double x, double y) {
        if (y == 0.0) return 1.0;
        if (x != x || y != y) return __longlong_as_double(0x7ff8000000000000LL);
        if (x == 0.0) return y > 0.0 ? 0.0 : __longlong_as_double(0x7ff0000000000000LL);
        if (x == 1.0) return 1.0;
        return pm_exp(y * pm_log(x));
    }
    __device__ static __forceinline__ double exp_(double x) { return pm_exp(x); }
};
struct MathF {
    __device__ static __forceinline__ void sincos_(float x, float &s, float &c) { __sincosf(x, &s, &c); }
    __device__ static __forceinline__ float pow_(float x, float y) {
        if (y == 0.0f) return 1.0f;
        if (x == 0.0f) return y > 0.0f ? 0.0f : __int_as_float(0x7f800000);
        return exp2f(y * __log2f(x));
    }
    __device__ static __forceinline__ float exp_(float x) { return __expf(x); }
};
template <typename T> struct Math;
template <> struct Math<double> : MathD {};
template <> struct Math<float> : MathF {};

// x^5 as x2*x2*x (Schlick's (1-cos)^5)
template <typename T> __device__ __forceinline__ T pow5(T x) { T x2 = x * x; T x4 = x2 * x2; return x4 * x; }

// ---------------------------------------------------------------------------
// Device scene tables (converted from the ABI structs to precision T)
// ---------------------------------------------------------------------------
template <typename T>
struct alignas(16) DObject {
    int32_t shape, mat;
    T p[3], n[3], d1[3], d2[3];
    T dist, radius;
};
static_assert(sizeof(DObject<float>) == 64, "FP32 object = four 16-byte vectors");
static_assert(sizeof(DObject<double>) == 128, "FP64 object = eight 16-byte vectors");

// object fetch with 16-byte vector loads (the table is read by every lane
// for every ray, uniformly: each load is one broadcast transaction).  Plain
// loads, not __ldg: the eye levels point the table at a copy in shared
// memory (eye_level), which the non-coherent global path cannot read.
template <typename T>
__device__ __forceinline__ DObject<T> load_object(const DObject<T> *objs, int i) {
    constexpr int NV = sizeof(DObject<T>) / 16;
    union {
        uint4 v[NV];
        DObject<T> o;
    } u;
    const uint4 *src = reinterpret_cast<const uint4 *>(objs + i);
#pragma unroll
    for (int k = 0; k < NV; k++) u.v[k] = src[k];
    return u.o;
}

template <typename T>
struct DMaterial {
    T emit[3];
    T ior[3];
    T cdiff[3], cspec[3];
    T scatter, metal, rough, dpow;
    int32_t surface;
    uint32_t flags;   // bit0 spec == BLACK, bit1 spec == WHITE, bit2 diff == BLACK
};

template <typename T>
struct DLight {
    int32_t kind, pad;
    T color[3];
    T flux;
    T pos[3], nvec[3], d1[3], d2[3], dir[3];
};

template <typename T>
struct DCamera {
    T eye[3], origin[3], esx[3], esy[3], eex[3], eey[3];
    T ambient[3];   // added to the direct light by the classic tracer
    int32_t xreso, yreso, jitter_aa, blur;
};

struct BvhNode;

// Scene tables of one precision.  With a hierarchy (bvh != nullptr) the
// bounded objects are reached through it and the unbounded ones (infinite
// planes) are listed in unb; without one every object is tested.
template <typename T, bool HAS_BVH = false>
struct SceneView {
    const DObject<T> *objs;
    const DMaterial<T> *mats;
    const DLight<T> *lights;
    int32_t n_objs, n_mats, n_lights;
    int32_t bvh_root;          // root node (>= 0), or ~object when one object is bounded
    const BvhNode *bvh;
    const int32_t *bvh_order;  // objects in Morton order (leaves are runs of it)
    const int32_t *unb;
    int32_t n_unb;
    int32_t bvh_steps;         // bound on one walk: 2 * objects in the tree + 64
    int32_t bvh_runs;          // leaves are runs of bvh_order (leaf size > 1)
    int32_t pad;
};

// the same tables typed for the kernels that walk the hierarchy
template <typename T>
__host__ __device__ inline SceneView<T, true> with_bvh(const SceneView<T, false> &v) {
    return SceneView<T, true>{v.objs, v.mats, v.lights, v.n_objs, v.n_mats, v.n_lights, v.bvh_root,
                              v.bvh, v.bvh_order, v.unb, v.n_unb, v.bvh_steps, v.bvh_runs, 0};
}

// Emission bookkeeping (src/bin/ppmpa.rs:30-31): light l owns emission
// indices [first[l], first[l+1]).
struct EmitPlan {
    int64_t first[17];
    int32_t n_lights;
    int32_t pad;
};

}  // namespace ppm
