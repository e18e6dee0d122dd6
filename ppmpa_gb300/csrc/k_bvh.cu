// k_bvh.cu -- linear BVH over the scene's bounded objects, built on the GPU.
//
//   1. bounds: FP64 box of every bounded object (sphere, triangle,
//      parallelogram), rounded outwards to FP32 and padded; its centroid;
//   2. centroid bounds (block reduction + one atomic per block);
//   3. 30-bit Morton code of each centroid (10 bits per axis);
//   4. stable LSD radix sort of (code, position) in four 8-bit passes;
//   5. hierarchy: Karras, "Maximizing parallelism in the construction of
//      BVHs, octrees and k-d trees" (HPG 2012) -- node i finds its key range
//      and split from the longest common prefixes of the sorted codes
//      (ties between equal codes broken by position); a child whose range
//      holds at most leaf_max (1..8) objects becomes a leaf run;
//   6. refit bottom-up: of the two threads supplying a node's child boxes
//      the second (atomic counter) merges them and carries on to the
//      parent, so no thread ever waits.
// Layout of the nodes: ppm_bvh.cuh.
#include <algorithm>
#include <utility>

#include "ppm_launch.h"

namespace ppm {

namespace {

constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ITEMS = 16;
constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ITEMS;

__device__ __forceinline__ float round_down(double x) { return __double2float_rd(x); }
__device__ __forceinline__ float round_up(double x) { return __double2float_ru(x); }

// 2^-17 of the coordinate magnitude (at least of 1): covers the rounding of
// the objects' own distance routines, so a box never cuts off a hit
__device__ __forceinline__ float pad_of(double lo, double hi) {
    double m = fmax(1.0, fmax(fabs(lo), fabs(hi)));
    return (float)(m * 7.62939453125e-6);
}

__global__ void k_bvh_bounds(const DObject<double> *objs, const int32_t *bounded, int m, float4 *blo, float4 *bhi,
                             float4 *centroid) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const DObject<double> o = load_object(objs, bounded[k]);
    double lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        if (o.shape == SH_SPHERE) {
            lo[a] = o.p[a] - o.radius;
            hi[a] = o.p[a] + o.radius;
        } else {
            double p0 = o.p[a], p1 = o.p[a] + o.d1[a], p2 = o.p[a] + o.d2[a];
            lo[a] = fmin(p0, fmin(p1, p2));
            hi[a] = fmax(p0, fmax(p1, p2));
            if (o.shape == SH_PARALLELOGRAM) {
                double p3 = (o.p[a] + o.d1[a]) + o.d2[a];
                lo[a] = fmin(lo[a], p3);
                hi[a] = fmax(hi[a], p3);
            }
        }
    }
    float l[3], h[3];
    for (int a = 0; a < 3; a++) {
        float pad = pad_of(lo[a], hi[a]);
        l[a] = round_down(lo[a]) - pad;
        h[a] = round_up(hi[a]) + pad;
    }
    blo[k] = make_float4(l[0], l[1], l[2], 0.0f);
    bhi[k] = make_float4(h[0], h[1], h[2], 0.0f);
    centroid[k] = make_float4(0.5f * (l[0] + h[0]), 0.5f * (l[1] + h[1]), 0.5f * (l[2] + h[2]), 0.0f);
}

// order-preserving float <-> uint for atomicMin / atomicMax
__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_bvh_init_bounds(uint32_t *cb) {
    if (threadIdx.x < 3) cb[threadIdx.x] = 0xffffffffu;          // min of encoded values
    else if (threadIdx.x < 6) cb[threadIdx.x] = 0u;              // max
}

__global__ void __launch_bounds__(256) k_bvh_centroid_bounds(const float4 *centroid, int m, uint32_t *cb) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        float4 c = centroid[k];
        lo[0] = fminf(lo[0], c.x); lo[1] = fminf(lo[1], c.y); lo[2] = fminf(lo[2], c.z);
        hi[0] = fmaxf(hi[0], c.x); hi[1] = fmaxf(hi[1], c.y); hi[2] = fmaxf(hi[2], c.z);
    }
    __shared__ float sl[3][8], sh[3][8];
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
        if ((threadIdx.x & 31) == 0) { sl[a][threadIdx.x >> 5] = lo[a]; sh[a][threadIdx.x >> 5] = hi[a]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int a = threadIdx.x;
        float l = INFINITY, h = -INFINITY;
        for (int w = 0; w < 8; w++) { l = fminf(l, sl[a][w]); h = fmaxf(h, sh[a][w]); }
        atomicMin(&cb[a], f2o(l));
        atomicMax(&cb[3 + a], f2o(h));
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_bvh_morton(const float4 *centroid, int m, const uint32_t *cb, uint32_t *code, uint32_t *pos) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    float4 c = centroid[k];
    float v[3] = {c.x, c.y, c.z};
    uint32_t q[3];
    for (int a = 0; a < 3; a++) {
        float lo = o2f(cb[a]), hi = o2f(cb[3 + a]);
        float ext = hi - lo;
        float t = ext > 0.0f ? (v[a] - lo) / ext : 0.0f;
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        q[a] = (uint32_t)fminf(t * 1024.0f, 1023.0f);
    }
    code[k] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    pos[k] = (uint32_t)k;
}

// ---- stable LSD radix sort, 8 bits per pass -------------------------------
__global__ void __launch_bounds__(RADIX_THREADS) k_radix_hist(const uint32_t *keys, int m, int shift, uint32_t *hist,
                                                             int nb) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ITEMS; r++) {
        int i = base + r * RADIX_THREADS + threadIdx.x;
        if (i < m) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of n counts in one block (n <= a few million)
__global__ void __launch_bounds__(1024) k_radix_scan(uint32_t *a, int n) {
    __shared__ uint32_t ws[32];
    const int per = (n + 1023) / 1024;
    const int b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (int j = 0; j < per; j++) {
        int i = b0 + j;
        if (i < n) s += a[i];
    }
    uint32_t incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if ((threadIdx.x & 31) >= (unsigned)o) incl += u;
    }
    if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t w = ws[threadIdx.x], wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, wi, o);
            if (threadIdx.x >= (unsigned)o) wi += u;
        }
        ws[threadIdx.x] = wi - w;
    }
    __syncthreads();
    uint32_t run = ws[threadIdx.x >> 5] + incl - s;
    for (int j = 0; j < per; j++) {
        int i = b0 + j;
        if (i < n) {
            uint32_t v = a[i];
            a[i] = run;
            run += v;
        }
    }
}

// Each block scatters its tile in RADIX_ITEMS rounds of 256 consecutive
// keys; inside a round a key's rank among equal digits comes from the warp
// (match_any) and the warps before it, so the pass is stable.
__global__ void __launch_bounds__(RADIX_THREADS) k_radix_scatter(const uint32_t *kin, const uint32_t *vin,
                                                                uint32_t *kout, uint32_t *vout, int m, int shift,
                                                                const uint32_t *hist, int nb) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[RADIX_THREADS / 32][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    base[threadIdx.x] = hist[threadIdx.x * nb + blockIdx.x];
    const int tile = blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ITEMS; r++) {
        for (int k = threadIdx.x; k < (RADIX_THREADS / 32) * 256; k += RADIX_THREADS) (&wcnt[0][0])[k] = 0;
        __syncthreads();
        const int i = tile + r * RADIX_THREADS + threadIdx.x;
        const bool valid = i < m;
        const uint32_t key = valid ? kin[i] : 0u;
        const uint32_t d = valid ? (key >> shift) & 255u : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned below = peers & ((1u << lane) - 1u);
        if (valid && below == 0u) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = base[d] + __popc(below);
            for (int w = 0; w < warp; w++) off += wcnt[w][d];
            kout[off] = key;
            vout[off] = vin[i];
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < RADIX_THREADS / 32; w++) add += wcnt[w][threadIdx.x];
        base[threadIdx.x] += add;
        __syncthreads();
    }
}

// ---- hierarchy (Karras 2012) -------------------------------------------------
__device__ __forceinline__ int delta(const uint32_t *code, int m, int i, int j) {
    if (j < 0 || j >= m) return -1;
    uint32_t a = code[i], b = code[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// Children whose key range holds at most leaf_max objects become leaves:
// ~(first << 3 | (count - 1)), a run of the Morton-ordered object list.
// Internal nodes inside such runs stay unreachable (parent -1).
__global__ void k_bvh_karras(const uint32_t *code, const int32_t *order, int m, int leaf_max, BvhNode *nodes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m - 1) return;
    const int d = delta(code, m, i, i + 1) > delta(code, m, i, i - 1) ? 1 : -1;
    const int dmin = delta(code, m, i, i - d);
    int lmax = 2;
    while (delta(code, m, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(code, m, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(code, m, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(code, m, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int g = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int nl = g - lo + 1, nr = hi - g;
    int left, right;
    // one object per leaf: the leaf is ~object itself (no indirection)
    if (nl <= leaf_max) left = leaf_max == 1 ? ~order[lo] : ~((lo << 3) | (nl - 1));
    else { left = g; nodes[g].d.z = i; nodes[g].d.w = 0; }
    if (nr <= leaf_max) right = leaf_max == 1 ? ~order[g + 1] : ~(((g + 1) << 3) | (nr - 1));
    else { right = g + 1; nodes[g + 1].d.z = i; nodes[g + 1].d.w = 1; }
    nodes[i].d.x = left;
    nodes[i].d.y = right;
    if (i == 0) { nodes[0].d.z = -1; nodes[0].d.w = 0; }
}

// order[k]: the object at sorted position k; inv_order[object]: its position
__global__ void k_bvh_order(const uint32_t *pos, const int32_t *bounded, int m, int32_t *order, int32_t *inv_order) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) {
        order[k] = bounded[pos[k]];
        inv_order[bounded[pos[k]]] = k;
    }
}

__device__ __forceinline__ void put_box(BvhNode &n, bool right, float4 lo, float4 hi) {
    if (!right) {
        n.a.x = lo.x; n.a.y = hi.x; n.a.z = lo.y; n.a.w = hi.y;
        n.c.x = lo.z; n.c.y = hi.z;
    } else {
        n.b.x = lo.x; n.b.y = hi.x; n.b.z = lo.y; n.b.w = hi.y;
        n.c.z = lo.z; n.c.w = hi.z;
    }
}

__device__ __forceinline__ void leaf_box(const uint32_t *pos, const float4 *blo, const float4 *bhi, int enc,
                                         int leaf_max, const int32_t *inv_order, float4 &lo, float4 &hi) {
    const int r = ~enc;
    const int first = leaf_max == 1 ? inv_order[r] : r >> 3, n = leaf_max == 1 ? 1 : (r & 7) + 1;
    lo = blo[pos[first]];
    hi = bhi[pos[first]];
    for (int k = 1; k < n; k++) {
        const float4 a = blo[pos[first + k]], b = bhi[pos[first + k]];
        lo = make_float4(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z), 0.0f);
        hi = make_float4(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z), 0.0f);
    }
}

// Bottom-up boxes.  Thread i writes the boxes of node i's leaf children;
// whichever thread supplies a node's second child box completes it (union
// of the two) and carries that box to the parent's slot (side d.w), so no
// thread waits for another.
__global__ void k_bvh_refit(const uint32_t *pos, const float4 *blo, const float4 *bhi, int m, int leaf_max,
                            const int32_t *inv_order, BvhNode *nodes, uint32_t *visits) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m - 1) return;
    const int4 d0 = nodes[i].d;
    uint32_t r = 0;
    float4 lo, hi;
    if (d0.x < 0) { leaf_box(pos, blo, bhi, d0.x, leaf_max, inv_order, lo, hi); put_box(nodes[i], false, lo, hi); r++; }
    if (d0.y < 0) { leaf_box(pos, blo, bhi, d0.y, leaf_max, inv_order, lo, hi); put_box(nodes[i], true, lo, hi); r++; }
    if (r == 0) return;
    __threadfence();
    int p = i;
    uint32_t add = r;
    for (;;) {
        if (atomicAdd(&visits[p], add) + add < 2u) return;   // the other child's thread completes p
        __threadfence();
        const float4 a = __ldcg(&nodes[p].a), b = __ldcg(&nodes[p].b), c = __ldcg(&nodes[p].c);
        lo = make_float4(fminf(a.x, b.x), fminf(a.z, b.z), fminf(c.x, c.z), 0.0f);
        hi = make_float4(fmaxf(a.y, b.y), fmaxf(a.w, b.w), fmaxf(c.y, c.w), 0.0f);
        const int4 dp = __ldcg(&nodes[p].d);
        if (dp.z < 0) return;                                 // the root, or a node inside a leaf run
        put_box(nodes[dp.z], dp.w != 0, lo, hi);
        __threadfence();
        p = dp.z;
        add = 1;
    }
}

}  // namespace

int bvh_scratch_words(int m, int n_objs) {
    const int nb = (m + RADIX_TILE - 1) / RADIX_TILE;
    // blo, bhi, centroid (4 words each), code x2, pos x2, hist, visits, bounds;
    // inv_order (one word per scene object, n_objs >= m) comes after
    return 12 * m + 4 * m + 256 * nb + m + 8 + n_objs;
}

int launch_bvh_build(const DObject<double> *objs, const int32_t *bounded, int m, int n_objs, int leaf_max,
                     BvhNode *nodes, int32_t *order, uint32_t *scratch, cudaStream_t s) {
    const int nb = (m + RADIX_TILE - 1) / RADIX_TILE;
    float4 *blo = (float4 *)scratch;
    float4 *bhi = blo + m;
    float4 *cen = bhi + m;
    uint32_t *code = (uint32_t *)(cen + m), *code2 = code + m, *pos = code2 + m, *pos2 = pos + m;
    uint32_t *hist = pos2 + m;
    uint32_t *visits = hist + 256 * nb;
    uint32_t *cb = visits + m;
    int32_t *inv_order = (int32_t *)(cb + 8);   // n_objs words
    const int g = (m + 255) / 256;
    k_bvh_bounds<<<g, 256, 0, s>>>(objs, bounded, m, blo, bhi, cen);
    k_bvh_init_bounds<<<1, 32, 0, s>>>(cb);
    k_bvh_centroid_bounds<<<std::min(g, 1024), 256, 0, s>>>(cen, m, cb);
    k_bvh_morton<<<g, 256, 0, s>>>(cen, m, cb, code, pos);
    for (int shift = 0; shift < 32; shift += 8) {
        k_radix_hist<<<nb, RADIX_THREADS, 0, s>>>(code, m, shift, hist, nb);
        k_radix_scan<<<1, 1024, 0, s>>>(hist, 256 * nb);
        k_radix_scatter<<<nb, RADIX_THREADS, 0, s>>>(code, pos, code2, pos2, m, shift, hist, nb);
        std::swap(code, code2);
        std::swap(pos, pos2);
    }
    k_bvh_order<<<g, 256, 0, s>>>(pos, bounded, m, order, inv_order);
    if (m <= leaf_max) return leaf_max == 1 ? ~bounded[0] : ~(m - 1);   // one leaf: the whole run
    cudaMemsetAsync(nodes, 0xff, sizeof(BvhNode) * (size_t)(m - 1), s);   // parents -1 until linked
    cudaMemsetAsync(visits, 0, sizeof(uint32_t) * m, s);
    k_bvh_karras<<<(m - 1 + 255) / 256, 256, 0, s>>>(code, order, m, leaf_max, nodes);
    k_bvh_refit<<<(m - 1 + 255) / 256, 256, 0, s>>>(pos, blo, bhi, m, leaf_max, inv_order, nodes, visits);
    return 0;
}

}  // namespace ppm
