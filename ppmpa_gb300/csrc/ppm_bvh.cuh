// ppm_bvh.cuh -- bounding-volume hierarchy over the scene's bounded objects.
//
// The reference intersects every object for every ray (calc_intersection,
// src/tracer.rs:306-350: the nearest t >= NEARLY0, the first object in list
// order among equal t).  Large scenes (a 1M-triangle mesh) need a hierarchy;
// the one here is a linear BVH (Karras 2012) built on the GPU (k_bvh.cu),
// and traversal keeps the reference's answer exactly: every object whose t
// can be <= the best t so far is tested, and ties go to the lower index.
//
// Node layout (one internal node = 64 bytes, both children's boxes, so one
// node fetch tests two boxes):
//   a = (L.lo.x, L.hi.x, L.lo.y, L.hi.y)
//   b = (R.lo.x, R.hi.x, R.lo.y, R.hi.y)
//   c = (L.lo.z, L.hi.z, R.lo.z, R.hi.z)
//   d = (left, right, parent, side)  child >= 0: internal node; < 0: a leaf:
//       ~object with one object per leaf, else ~(first << 3 | (count - 1)),
//       objects order[first .. first + count) of the Morton-ordered list
// Boxes are FP32, rounded outwards from the FP64 object bounds and padded by
// 2^-17 of the coordinate magnitude, so the same tree serves the FP64 and
// the FP32 tracers and a box never excludes a hit its object's own distance
// routine reports at or below the best t.
#pragma once
#include "ppm_common.cuh"

namespace ppm {

struct BvhNode {
    float4 a, b, c;
    int4 d;
};

// Deepest traversal stack: the tree's depth is bounded by its key length,
// 30 Morton bits + 31 index bits in the worst case of all-equal codes; real
// scenes stay far below 64.
constexpr int BVH_STACK = 64;

template <typename T> struct BoxMath;
template <> struct BoxMath<float> {
    __device__ static __forceinline__ float tiny() { return 1e-20f; }
};
template <> struct BoxMath<double> {
    __device__ static __forceinline__ double tiny() { return 1e-30; }
};

// slab test of the ray (o, inv = 1/d) against [lo, hi]; [t0, t1] the overlap
template <typename T>
__device__ __forceinline__ void slab(T o, T inv, float lo, float hi, T &t0, T &t1) {
    T a = ((T)lo - o) * inv, b = ((T)hi - o) * inv;
    t0 = a < b ? a : b;
    t1 = a < b ? b : a;
}
// FP32: o is passed as o * inv, so each bound is one fused multiply-add
// (lo * inv - o * inv); the few-ulp difference from (lo - o) * inv near the
// origin is far inside the boxes' 2^-17 outward padding.
__device__ __forceinline__ void slab(float oinv, float inv, float lo, float hi, float &t0, float &t1) {
    const float a = __fmaf_rn(lo, inv, -oinv), b = __fmaf_rn(hi, inv, -oinv);   // finite: inv clamped by safe_inv
    t0 = fminf(a, b);
    t1 = fmaxf(a, b);
}

// o: the ray origin (FP64), or origin * inv (FP32, see slab)
template <typename T>
__device__ __forceinline__ bool box_hit(V3<T> o, V3<T> inv, float lx, float hx, float ly, float hy, float lz, float hz,
                                        T tmax, T &tnear) {
    T x0, x1, y0, y1, z0, z1;
    slab(o.x, inv.x, lx, hx, x0, x1);
    slab(o.y, inv.y, ly, hy, y0, y1);
    slab(o.z, inv.z, lz, hz, z0, z1);
    T tn, tf;
    if constexpr (sizeof(T) == 4) {
        tn = fmaxf(fmaxf(x0, y0), z0);
        tf = fminf(fminf(x1, y1), z1);
    } else {
        tn = x0 > y0 ? x0 : y0;
        tn = tn > z0 ? tn : z0;
        tf = x1 < y1 ? x1 : y1;
        tf = tf < z1 ? tf : z1;
    }
    tnear = tn;
    return tn <= tf && tf >= Cst<T>::nearly0() && tn <= tmax;
}

template <typename T>
__device__ __forceinline__ T safe_inv(T d) {
    T a = d < T(0) ? -d : d;
    if (a < BoxMath<T>::tiny()) d = d < T(0) ? -BoxMath<T>::tiny() : BoxMath<T>::tiny();
    return T(1) / d;
}

// Walks the tree rooted at `root` calling test(object) for every object whose
// box the ray meets no farther than best(); test() may lower best().  One
// node or one leaf per step (an "if-if" walk: on these scenes it ran faster
// than a while-while walk, which serialises a warp's node and leaf phases).
// A walk visits each of the 2m - 1 nodes at most once; max_steps (2m + 64)
// bounds it even for a malformed tree.  runs: leaves are runs of `order`
// (leaf size > 1); otherwise a leaf is ~object.
template <typename T, typename Test, typename Best>
__device__ __forceinline__ void bvh_walk(const BvhNode *nodes, const int32_t *order, bool runs, int root,
                                         int max_steps, V3<T> o, V3<T> dir, Test &&test, Best &&best) {
    const V3<T> inv = mk3(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
    if constexpr (sizeof(T) == 4) o = mk3(o.x * inv.x, o.y * inv.y, o.z * inv.z);   // the slabs' form
    int stack[BVH_STACK];
    int sp = 0;
    int node = root;
    for (int step = 0; step < max_steps; step++) {
        if (node < 0) {
            if (runs) {
                const int r = ~node, first = r >> 3, n = (r & 7) + 1;
                for (int k = 0; k < n; k++) test(__ldg(&order[first + k]));
            } else {
                test(~node);
            }
        } else {
            const float4 a = __ldg(&nodes[node].a), b = __ldg(&nodes[node].b), c = __ldg(&nodes[node].c);
            const int4 d = __ldg(&nodes[node].d);
            const T tb = best();
            T tl, tr;
            const bool hl = box_hit(o, inv, a.x, a.y, a.z, a.w, c.x, c.y, tb, tl);
            const bool hr = box_hit(o, inv, b.x, b.y, b.z, b.w, c.z, c.w, tb, tr);
            if (hl && hr) {
                const bool lf = tl <= tr;
                if (sp < BVH_STACK) stack[sp++] = lf ? d.y : d.x;
                node = lf ? d.x : d.y;
                continue;
            }
            if (hl) { node = d.x; continue; }
            if (hr) { node = d.y; continue; }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
}

}  // namespace ppm
