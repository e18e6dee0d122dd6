// ppm_trace.cuh -- intersection, surface sampling, lights, the photon bounce
// event and the eye-vertex evaluation, templated on the arithmetic type T
// (double: plain path, float: mixed path).  Each function cites the
// reference function whose semantics it implements.
#pragma once
#include "ppm_common.cuh"

namespace ppm {

template <typename T> struct Cst {
    __device__ static constexpr T nearly0() { return T(NEARLY0); }
    __device__ static constexpr T pi() { return T(PI_D); }
    __device__ static constexpr T one_pi() { return T(ONE_PI_D); }
    __device__ static constexpr T sr_half() { return T(SR_HALF_D); }
    __device__ static constexpr T pi4() { return T(PI4_D); }
    __device__ static T inf() { return T(INFINITY); }
};

}  // namespace ppm

#include "ppm_bvh.cuh"

namespace ppm {

// ---------------------------------------------------------------------------
// Shapes: src/ray/geometry.rs:132-202
// ---------------------------------------------------------------------------
template <typename T> struct Div;
template <> struct Div<double> {   // FP64: true division, as the reference
    double inv;
    __device__ __forceinline__ explicit Div(double d) : inv(d) {}
    __device__ __forceinline__ double of(double x) const { return x / inv; }
};
template <> struct Div<float> {    // FP32: one reciprocal, three multiplies
    float inv;
    __device__ __forceinline__ explicit Div(float d) : inv(1.0f / d) {}
    __device__ __forceinline__ float of(float x) const { return x * inv; }
};

// Moller-Trumbore as method_moller (geometry.rs:149-165), with early exits:
// every value that decides the result is computed exactly as the reference
// computes it, so the FP64 outcome is unchanged.
template <typename T>
__device__ __forceinline__ bool method_moller(T l, V3<T> p0, V3<T> d1, V3<T> d2, V3<T> p, V3<T> d, T &t) {
    V3<T> re2 = cross(d, d2);
    T det_a = dot(re2, d1);
    if (det_a == T(0)) return false;
    Div<T> dv(det_a);
    V3<T> pp = p - p0;
    T u = dv.of(dot(re2, pp));
    if (u < T(0) || u > T(1)) return false;
    V3<T> te1 = cross(pp, d1);
    T v = dv.of(dot(te1, d));
    if (v < T(0) || v > T(1) || u + v > l) return false;
    t = dv.of(dot(te1, d2));
    return true;
}

// FP32: every product and sum rounded as written.  Left to the compiler,
// a cross product x*y - z*w contracts to fma(x, y, -z*w) or fma(-z, w, x*y)
// depending on the code around it, so two kernels that inline the test (a
// single render's trace and a batch's) could disagree in the last bit near
// an edge and send a ray to a neighbouring triangle.
__device__ __forceinline__ float dot_rn(V3<float> a, V3<float> b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
__device__ __forceinline__ V3<float> cross_rn(V3<float> a, V3<float> b) {
    return mk3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
               __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
template <>
__device__ __forceinline__ bool method_moller<float>(float l, V3<float> p0, V3<float> d1, V3<float> d2, V3<float> p,
                                                     V3<float> d, float &t) {
    const V3<float> re2 = cross_rn(d, d2);
    const float det_a = dot_rn(re2, d1);
    if (det_a == 0.0f) return false;
    const float inv = __frcp_rn(det_a);
    const V3<float> pp = mk3(__fsub_rn(p.x, p0.x), __fsub_rn(p.y, p0.y), __fsub_rn(p.z, p0.z));
    const float u = __fmul_rn(dot_rn(re2, pp), inv);
    if (u < 0.0f || u > 1.0f) return false;
    const V3<float> te1 = cross_rn(pp, d1);
    const float v = __fmul_rn(dot_rn(te1, d), inv);
    if (v < 0.0f || v > 1.0f || __fadd_rn(u, v) > l) return false;
    t = __fmul_rn(dot_rn(te1, d2), inv);
    return true;
}

template <typename T>
__device__ __forceinline__ int shape_distance(const DObject<T> &o, V3<T> rp, V3<T> rd, T &ta, T &tb) {
    switch (o.shape) {
    case SH_PLAIN: {
        V3<T> n = ld3(o.n);
        T cos0 = dot(n, rd);
        if (cos0 == T(0)) return 0;
        ta = (o.dist + dot(n, rp)) / -cos0;
        return 1;
    }
    case SH_SPHERE: {
        V3<T> oc = ld3(o.p) - rp;
        T t0 = dot(oc, rd);
        T t1 = o.radius * o.radius - (dot(oc, oc) - t0 * t0);
        if (t1 <= T(0)) return 0;
        T t2 = dsqrt(t1);
        if (t2 == T(0)) { ta = t0; return 1; }
        ta = t0 - t2; tb = t0 + t2;
        return 2;
    }
    case SH_POLYGON:
    case SH_PARALLELOGRAM: {
        T l = o.shape == SH_POLYGON ? T(1) : T(2);
        return method_moller(l, ld3(o.p), ld3(o.d1), ld3(o.d2), rp, rd, ta) ? 1 : 0;
    }
    default:
        return 0;
    }
}

template <typename T>
struct Isect {
    V3<T> pos, n;
    T t;
    int obj;
    bool in;
};

// calc_intersection, src/tracer.rs:306-350: nearest t >= NEARLY0, the first
// object in list order among equal t (stable sort); normal flipped to face
// the ray (io = Out when flipped).
template <typename T, bool B>
__device__ __forceinline__ bool intersect(const SceneView<T, B> &sc, V3<T> rp, V3<T> rd, Isect<T> &is) {
    T best = T(0);
    int bi = -1;
    if constexpr (!B) {
        for (int i = 0; i < sc.n_objs; i++) {
            T ta, tb;
            const DObject<T> o = load_object(sc.objs, i);
            int k = shape_distance(o, rp, rd, ta, tb);
            if (k >= 1 && ta >= Cst<T>::nearly0() && (bi < 0 || ta < best)) { best = ta; bi = i; }
            if (k == 2 && tb >= Cst<T>::nearly0() && (bi < 0 || tb < best)) { best = tb; bi = i; }
        }
    } else {
        // the list-order rule of the loop above, for any visiting order:
        // smallest t, then smallest index
        auto test = [&](int i) {
            T ta, tb;
            const DObject<T> o = load_object(sc.objs, i);
            int k = shape_distance(o, rp, rd, ta, tb);
            if (k >= 1 && ta >= Cst<T>::nearly0() && (bi < 0 || ta < best || (ta == best && i < bi))) {
                best = ta;
                bi = i;
            }
            if (k == 2 && tb >= Cst<T>::nearly0() && (bi < 0 || tb < best || (tb == best && i < bi))) {
                best = tb;
                bi = i;
            }
        };
        for (int k = 0; k < sc.n_unb; k++) test(sc.unb[k]);
        bvh_walk<T>(sc.bvh, sc.bvh_order, sc.bvh_runs != 0, sc.bvh_root, sc.bvh_steps, rp, rd, test,
                    [&]() { return bi < 0 ? Cst<T>::inf() : best; });
    }
    if (bi < 0) return false;
    const DObject<T> o = load_object(sc.objs, bi);
    V3<T> p = rp + rd * best;
    V3<T> n;
    if (o.shape == SH_SPHERE) {
        if (!normalize(p - ld3(o.p), n)) return false;
    } else if (o.shape == SH_POINT) {
        return false;
    } else {
        n = ld3(o.n);
    }
    if (dot(n, rd) > T(0)) { is.n = -n; is.in = false; }
    else { is.n = n; is.in = true; }
    is.pos = p; is.obj = bi; is.t = best;
    return true;
}

// ---------------------------------------------------------------------------
// Physics: src/ray/physics.rs:200-335, surface.rs:408-417, algebra.rs:211-235
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T relative_ior(T a, T b) { return a == T(0) ? T(1) : b / a; }

template <typename T>
__device__ __forceinline__ T relative_ior_average(const T *i1, const T *i2) {
    T a1 = (i1[0] + i1[1] + i1[2]) / T(3);
    T a2 = (i2[0] + i2[1] + i2[2]) / T(3);
    return relative_ior(a1, a2);
}

template <typename T> __device__ __forceinline__ T schlick(T f0, T cos) { return f0 + (T(1) - f0) * pow5(T(1) - cos); }

template <typename T> __device__ __forceinline__ int rr1(Rng &r, T p0) {
    T p = gen_range<T>(r, T(0), T(1));
    return p > p0 ? 1 : 0;
}

template <typename T>
__device__ __forceinline__ V3<T> specular_reflection(V3<T> n, V3<T> v, T &cos_out) {
    T cos = -dot(v, n);
    if (cos < T(0)) { cos_out = -cos; return n; }
    V3<T> r = n;
    normalize(v + (T(2) * cos) * n, r);
    cos_out = cos;
    return r;
}

template <typename T>
__device__ __forceinline__ bool specular_refraction(V3<T> n, V3<T> v, T eta, V3<T> &t_out, T &cos2) {
    T cos1 = -dot(v, n);
    if (cos1 < T(0)) { cos2 = T(0); return false; }
    T sq_eta = eta * eta;
    T sq_cos = cos1 * cos1;
    T g0 = sq_eta + sq_cos - T(1);
    // eta = 0 (a surface without an IOR) leaves g0 <= 0 except where
    // rounding makes |cos1| reach 1: there the reference divides g by 0
    // (0/0 or x/0) and the weights become NaN; no refraction instead
    if (g0 < T(0) || eta == T(0)) { cos2 = T(0); return false; }
    T g = dsqrt(g0);
    cos2 = g / eta;
    return normalize((T(1) / eta) * (v + (cos1 - g) * n), t_out);
}

// reflection_glossy, physics.rs:232-261 (two draws)
template <typename T>
__device__ __forceinline__ V3<T> reflection_glossy(Rng &rg, V3<T> n, V3<T> r, T pw) {
    V3<T> u = mk3(T(1), T(0), T(0));
    if (!normalize(cross(mk3(T(0.00424), T(1), T(0.00764)), r), u))
        normalize(cross(mk3(T(1), T(0.00424), T(0.00764)), r), u);
    V3<T> v = cross(u, r);
    // r is a reflection about n, so n.r >= 0; at grazing incidence rounding
    // can make it a hair negative, where xi0^(pw n.r) > 1 and the square
    // root below is NaN (in the reference too): clamped to 0
    T c0 = dot(n, r);
    if (c0 < T(0)) c0 = T(0);
    T xi0 = gen_range<T>(rg, T(0), T(1));
    T xi1 = Math<T>::pow_(xi0, pw * c0);
    T xi2 = T(2.0 * PI_D) * gen_range<T>(rg, T(0), T(1));
    T sq = dsqrt(T(1) - xi1 * xi1);
    T sn, cs;
    Math<T>::sincos_(xi2, sn, cs);
    T x = cs * sq;
    T y = xi1;
    T z = sn * sq;
    V3<T> wi = (x * u + y * r) + z * v;
    if (dot(n, wi) < T(0)) wi = ((-x) * u + y * r) - z * v;
    V3<T> out = mk3(T(1), T(0), T(0));
    normalize(wi, out);
    return out;
}

// generate_random_dir_by_angle + diffuse_reflection (two draws)
template <typename T>
__device__ __forceinline__ V3<T> diffuse_reflection(Rng &rg, V3<T> n) {
    T phi = gen_range<T>(rg, T(0), T(2.0 * PI_D));
    T xi = gen_range<T>(rg, T(-1), T(1));
    T xi2 = dsqrt(T(1) - xi * xi);
    T sn, cs;
    Math<T>::sincos_(phi, sn, cs);
    V3<T> d = mk3(T(0), T(1), T(0));
    normalize(mk3(xi2 * cs, xi, xi2 * sn), d);
    return dot(n, d) > T(0) ? d : -d;
}

// generate_random_dir (cube rejection, 3 draws per trial, at most 256 trials).
// The FP32 path draws the same uniform distribution on the sphere directly
// (z = 1 - 2u, phi = 2 pi v: Archimedes' hat-box theorem), two draws and no
// loop: the rejection loop's trial count differs between the lanes of a
// warp, and the warp waits for its slowest lane.  The FP64 path keeps the
// reference's draws, which its parity with the oracle checks one by one.
template <typename T>
__device__ __forceinline__ V3<T> random_dir(Rng &rg) {
    if constexpr (sizeof(T) == 4) {
        const T z = gen_range<T>(rg, T(-1), T(1));
        const T phi = gen_range<T>(rg, T(0), T(2.0 * PI_D));
        const T r = dsqrt(fmaxf(T(1) - z * z, T(0)));
        T sn, cs;
        Math<T>::sincos_(phi, sn, cs);
        return mk3(r * cs, r * sn, z);
    }
    for (int it = 0; it < 256; it++) {
        T x = gen_range<T>(rg, T(-1), T(1));
        T y = gen_range<T>(rg, T(-1), T(1));
        T z = gen_range<T>(rg, T(-1), T(1));
        V3<T> v = mk3(x, y, z);
        T len = dsqrt(dot(v, v));
        if (T(0) < len && len <= T(1)) {
            V3<T> o = v;
            normalize(v, o);
            return o;
        }
    }
    return mk3(T(0), T(1), T(0));
}

// ---------------------------------------------------------------------------
// Surfaces: src/ray/surface.rs
// ---------------------------------------------------------------------------
enum { MF_SPEC_BLACK = 1, MF_SPEC_WHITE = 2, MF_DIFF_BLACK = 4 };

template <typename T> __device__ __forceinline__ bool sf_reflect(const DMaterial<T> &m, T cos) {
    if (m.surface == SF_SIMPLE) return !(m.scatter == T(1) || (cos == T(1) && (m.flags & MF_SPEC_BLACK)));
    if (m.surface == SF_TS) {
        if (m.metal == T(0)) return true;
        if (m.metal == T(1)) return !(m.flags & MF_SPEC_BLACK);
        return true;
    }
    return false;
}
template <typename T> __device__ __forceinline__ bool sf_refract(const DMaterial<T> &m, T cos) {
    if (m.surface == SF_SIMPLE) return !(cos == T(0) && (m.flags & MF_SPEC_WHITE));
    if (m.surface == SF_TS) return m.metal == T(0) && m.scatter < T(1) && !(m.flags & MF_DIFF_BLACK);
    return false;
}
template <typename T> __device__ __forceinline__ bool sf_store(const DMaterial<T> &m) {
    if (m.surface == SF_SIMPLE) return m.scatter > T(0);
    if (m.surface == SF_TS) return m.metal != T(1) && m.scatter != T(0);
    return true;
}
template <typename T> __device__ __forceinline__ T sel(const T *c, int wl) { return wl == 0 ? c[0] : (wl == 1 ? c[1] : c[2]); }
template <typename T> __device__ __forceinline__ T sf_albedo_diff(const DMaterial<T> &m, int wl) {
    return (m.surface == SF_SIMPLE || m.surface == SF_TS) ? sel(m.cdiff, wl) : T(0);
}
template <typename T> __device__ __forceinline__ T sf_albedo_spec(const DMaterial<T> &m, int wl) {
    return (m.surface == SF_SIMPLE || m.surface == SF_TS) ? sel(m.cspec, wl) : T(0);
}
template <typename T> __device__ __forceinline__ T sf_roughness(const DMaterial<T> &m) {
    return m.surface == SF_SIMPLE ? m.scatter : (m.surface == SF_TS ? m.rough : T(0));
}
template <typename T> __device__ __forceinline__ T sf_power_glossy(const DMaterial<T> &m) {
    return (m.surface == SF_SIMPLE || m.surface == SF_TS) ? m.dpow : T(0);
}

// M_AIR (src/scene.rs:13-18): ior (1,1,1)
template <typename T, bool B>
__device__ __forceinline__ const T *ior_of(const SceneView<T, B> &sc, int m, const T *air) {
    return m < 0 ? air : sc.mats[m].ior;
}

// ---------------------------------------------------------------------------
// Photon emission: Light::generate_photon (light.rs:67-91)
// ---------------------------------------------------------------------------
template <typename T>
struct PhotonPath {
    V3<T> pos, dir;
    int wl, medium, level;
    uint32_t item;
};

// Spot light (no reference counterpart: the reference has point,
// parallelogram and sun lights, light.rs:16-38): a point light whose photons
// leave uniformly over the solid angle of the cone around axis a with
// cos(half-angle) cos_cut.  Two draws: u for cos(theta) = 1 - u (1 - cos_cut),
// then phi in [0, 2 pi); the frame is b1 = normalize(h x a), b2 = a x b1 with
// h = x unless |a.x| >= 0.9, then y.
template <typename T>
__device__ __forceinline__ V3<T> spot_dir(Rng &rg, V3<T> a, T cos_cut) {
    T u = gen_range<T>(rg, T(0), T(1));
    T phi = gen_range<T>(rg, T(0), T(2.0 * PI_D));
    T c = T(1) - u * (T(1) - cos_cut);
    T s = dsqrt(T(1) - c * c);
    T sn, cs;
    Math<T>::sincos_(phi, sn, cs);
    V3<T> h = (a.x < T(0) ? -a.x : a.x) < T(0.9) ? mk3(T(1), T(0), T(0)) : mk3(T(0), T(1), T(0));
    V3<T> b1 = mk3(T(1), T(0), T(0));
    normalize(cross(h, a), b1);
    V3<T> b2 = cross(a, b1);
    V3<T> d = a;
    normalize((b1 * (s * cs) + b2 * (s * sn)) + a * c, d);
    return d;
}

template <typename T>
__device__ __forceinline__ void generate_photon(const DLight<T> &l, Rng &rg, PhotonPath<T> &ph) {
    T p = gen_range<T>(rg, T(0), T(1));
    ph.wl = p < l.color[0] ? 0 : (p < l.color[0] + l.color[1] ? 1 : 2);
    if (l.kind == LT_POINT) {
        ph.pos = ld3(l.pos);
        ph.dir = random_dir<T>(rg);
    } else if (l.kind == LT_SPOT) {
        ph.pos = ld3(l.pos);
        ph.dir = spot_dir<T>(rg, ld3(l.dir), l.d1[0]);
    } else {
        T t1 = gen_range<T>(rg, T(0), T(1));
        T t2 = gen_range<T>(rg, T(0), T(1));
        if (l.kind == LT_PARALLELOGRAM) ph.dir = diffuse_reflection(rg, ld3(l.nvec));
        else ph.dir = ld3(l.dir);
        ph.pos = (ld3(l.pos) + t1 * ld3(l.d1)) + t2 * ld3(l.d2);
    }
    ph.medium = -1;
    ph.level = 0;
}

// One level of trace_photon (tracer.rs:31-125, surface.rs:211-258).
// Returns true if the path continues (ph updated); `store` / `spos` report
// whether the incoming photon is stored at this hit (tracer.rs:77-79).
template <typename T, bool B>
__device__ __forceinline__ bool photon_event(const SceneView<T, B> &sc, uint64_t seed, uint32_t pass, bool uc,
                                             PhotonPath<T> &ph, bool &store, V3<T> &spos) {
    store = false;
    Isect<T> is;
    if (!intersect(sc, ph.pos, ph.dir, is)) return false;
    const int mid = sc.objs[is.obj].mat;
    const DMaterial<T> &mate = sc.mats[mid];
    const T air[3] = {T(1), T(1), T(1)};
    Rng rg;
    rg.init<T>(seed, ph.item, pass, TAG_BOUNCE | (uint32_t)ph.level);
    bool cont = false;
    int nmed = ph.medium;
    V3<T> nd = ph.dir;
    if (mate.surface == SF_SIMPLE) {
        if (rr1<T>(rg, sf_roughness(mate)) == 0) {
            if (rr1<T>(rg, sf_albedo_diff(mate, ph.wl)) == 0) {
                nd = diffuse_reflection(rg, is.n);
                cont = true;
            }
        } else {
            T cos1;
            V3<T> rdir = specular_reflection(is.n, ph.dir, cos1);
            T f = schlick(sf_albedo_spec(mate, ph.wl), cos1);
            if (rr1<T>(rg, f) == 0) {
                nd = rdir; cont = true;
            } else if (sel(mate.ior, ph.wl) == T(0)) {
                // absorbed
            } else {
                T eta = relative_ior(sel(ior_of(sc, ph.medium, air), ph.wl), sel(mate.ior, ph.wl));
                T c2;
                V3<T> td;
                if (specular_refraction(is.n, ph.dir, eta, td, c2)) {
                    nmed = dot(td, is.n) < T(0) ? mid : -1;
                    nd = td; cont = true;
                }
            }
        }
    } else if (mate.surface == SF_TS) {
        T eta = relative_ior(sel(ior_of(sc, ph.medium, air), ph.wl), sel(mate.ior, ph.wl));
        T cos1, cos2;
        V3<T> rdir0 = specular_reflection(is.n, ph.dir, cos1);
        V3<T> rdir = reflection_glossy(rg, is.n, rdir0, sf_power_glossy(mate));
        V3<T> hvec = is.n, td;
        if (!normalize(rdir - ph.dir, hvec)) hvec = is.n;
        bool has_t = specular_refraction(hvec, ph.dir, eta, td, cos2);
        T cos = cos1 < cos2 ? cos1 : cos2;
        T f = schlick(sf_albedo_spec(mate, ph.wl), cos);
        if (rr1<T>(rg, f) == 0) {
            nd = rdir; cont = true;
        } else if (rr1<T>(rg, sf_albedo_diff(mate, ph.wl)) == 1) {
            // absorbed
        } else if (rr1<T>(rg, mate.scatter) == 0) {
            nd = diffuse_reflection(rg, is.n); cont = true;
        } else if (has_t) {
            nd = td; cont = true; nmed = mid;   // tracer.rs:68 keeps the hit material
        }
    }
    if ((!uc || ph.level > 0) && sf_store(mate)) { store = true; spos = is.pos; }
    if (!cont) return false;
    ph.pos = is.pos; ph.dir = nd; ph.medium = nmed;
    ph.level += 1;
    return ph.level < MAX_TRACE;
}

// ---------------------------------------------------------------------------
// Direct light (tracer.rs:263-290, light.rs:93-150), including the
// reference's shifted pairing of radiances and cosines (get_radiance prepends
// RADIANCE0, so sample k's cos^2 multiplies sample k-1's radiance and a
// single-sample light contributes nothing).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ V3<T> light_radiance(const DLight<T> &l, T d) {
    T l0;
    if (l.kind == LT_POINT || l.kind == LT_SPOT) l0 = l.flux / (Cst<T>::pi4() * d);
    else if (l.kind == LT_PARALLELOGRAM) l0 = (T(2) * l.flux * T(PARA_DIV) * T(PARA_DIV)) / (Cst<T>::pi4() * d);
    else l0 = l.flux;
    return mk3(l.color[0] * l0, l.color[1] * l0, l.color[2] * l0);
}

template <typename T, bool B>
__device__ __forceinline__ bool light_sample(const SceneView<T, B> &sc, V3<T> p, V3<T> n, V3<T> ld, T &dist2, T &cos2) {
    V3<T> ld3;
    if (!normalize(ld, ld3)) return false;
    T cos0 = dot(n, ld3);
    if (cos0 < T(0)) return false;
    Isect<T> is;
    if (!intersect(sc, p, ld3, is)) return false;
    T sq_ldist = dot(ld, ld);
    V3<T> dd = is.pos - p;
    T sq_odist = dot(dd, dd);
    if (sq_ldist - sq_odist > T(0.002)) return false;
    dist2 = sq_ldist; cos2 = cos0 * cos0;
    return true;
}

template <typename T, bool B>
__device__ __forceinline__ V3<T> radiance_from_light(const SceneView<T, B> &sc, V3<T> p, V3<T> n, const DLight<T> &l) {
    V3<T> rad = mk3(T(0), T(0), T(0));
    if (l.kind != LT_PARALLELOGRAM) return rad;   // at most one sample: contributes zero
    const T tss[5] = {T(0.1), T(0.3), T(0.5), T(0.7), T(0.9)};
    bool have_prev = false;
    T prev_d = T(0);
    for (int a = 0; a < 5; a++)
        for (int b = 0; b < 5; b++) {
            V3<T> sp = (ld3(l.pos) + tss[a] * ld3(l.d1)) + tss[b] * ld3(l.d2);
            V3<T> d = sp - p;
            if (!(dot(ld3(l.nvec), d) < T(0))) continue;
            T dist2, cos2;
            if (!light_sample(sc, p, n, d, dist2, cos2)) continue;
            V3<T> r = have_prev ? light_radiance(l, prev_d) : mk3(T(0), T(0), T(0));
            rad = rad + r * cos2;
            have_prev = true;
            prev_d = dist2;
        }
    return rad;
}

// ---------------------------------------------------------------------------
// Eye vertex coefficients: Surface::bsdf (surface.rs:135-206) is linear in
// (di, si, ti) with per-channel colour weights; the eye tree is evaluated as
// a sum over vertices of throughput x (emittance/(2 pi) + c_di * di).
// ---------------------------------------------------------------------------
template <typename T>
struct Coef {
    V3<T> di, si, ti;
};

template <typename T>
__device__ __forceinline__ V3<T> reflection_index(const T *col, T c) {
    T c2 = pow5(T(1) - c);
    return mk3(col[0] + (T(1) - col[0]) * c2, col[1] + (T(1) - col[1]) * c2, col[2] + (T(1) - col[2]) * c2);
}

template <typename T>
__device__ __forceinline__ Coef<T> bsdf_coef(const DMaterial<T> &m, T cos0) {
    Coef<T> c;
    V3<T> z = mk3(T(0), T(0), T(0));
    c.di = z; c.si = z; c.ti = z;
    if (m.surface == SF_SIMPLE) {
        V3<T> f = reflection_index(m.cspec, cos0);
        T d = m.scatter;
        c.di = mk3(d * (m.cdiff[0] * Cst<T>::one_pi()), d * (m.cdiff[1] * Cst<T>::one_pi()), d * (m.cdiff[2] * Cst<T>::one_pi()));
        c.si = (T(1) - d) * f;
        T om = (T(1) - d) * (T(1) - m.metal);
        c.ti = mk3(om * (T(1) - f.x), om * (T(1) - f.y), om * (T(1) - f.z));
    } else if (m.surface == SF_TS) {
        V3<T> f = reflection_index(m.cspec, cos0);
        if (m.metal == T(0)) {
            V3<T> fa = mk3((T(1) - f.x) * m.cdiff[0], (T(1) - f.y) * m.cdiff[1], (T(1) - f.z) * m.cdiff[2]);
            c.di = fa * (m.scatter * Cst<T>::one_pi());
            c.ti = fa * (T(1) - m.scatter);
        }
        c.si = f;
    }
    return c;
}

}  // namespace ppm
