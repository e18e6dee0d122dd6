// ppm_kernels.cuh -- the pass kernels, templated on the arithmetic type.
//
//   trace   : emission + bounce loop, one thread per photon path with path
//             regeneration; stored photons appended with warp-aggregated
//             atomics (tracer.rs:31-125, ppmpa.rs:86-92)
//   bbox    : bounds of the stored photons (grid extent)
//   hist    : cell key + rank per photon (counting-sort histogram)
//   scatter : photons moved into cell order (the photon map,
//             photonmap.rs:23-29 -- a sort-by-cell grid replaces the kd-tree)
//   eye     : camera rays + eye tree (tracer.rs:129-177) depth first with a
//             per-thread stack; throughput-weighted hit points appended
//   gather  : one warp per hit point scans the cell rows around it and sums
//             photon_to_radiance over the exact in-radius set (tracer.rs:179-195)
//   accum   : FP64 running sum of pass images (util/averager.rb:66-69)
#pragma once
#include <type_traits>
#include "ppm_trace.cuh"

namespace ppm {

// ---------------------------------------------------------------------------
// shared device state
// ---------------------------------------------------------------------------
// Photons are counting-sorted by key = 3 * cell + wavelength: the photons of
// a cell row are contiguous, and inside each cell they are grouped by
// wavelength (so a warp's flux updates mostly go to one channel).
// Cells are c wide in y and z and c / sx wide in x: a cell row (fixed y, z)
// is contiguous in the sorted map, and the finer x cells let a query's x
// range follow its sphere's chord closely while the number of rows stays
// (2 ext + 1)^2.
struct GridParams {
    double org[3];
    double cell, inv;         // y/z cell size c and 1/c
    double invx;              // 1 / (c / sx)
    float orgf[3];
    float invf, invxf;
    int32_t dim[3];
    int32_t ext, extx;        // cells a radius can span: y/z, x
    int64_t ncell;
    int64_t nkeys;            // map keys: one per cell
    float r2f, r2_lo, r2_hi;  // pass radius^2 in FP32 and its rounding band
    float cellf;              // cell size in FP32
};

struct PassState {
    double r2;                 // radius^2 used by the current pass
    double alpha;
    int32_t pass;              // random-stream pass index
    int32_t offset;            // PA schedule offset
    unsigned long long n_stored;
    unsigned long long n_hits;
    unsigned int overflow;     // bit0 photons, bit1 hit points, bit2 eye stack
    unsigned int pad;
    unsigned long long bb_lo[3], bb_hi[3];   // orderable encodings of f64 bounds
    GridParams grid;
    unsigned long long candidates, in_radius;   // gather counters (valid candidates, hits)
    unsigned long long slots, rows;             // lane slots issued, non-empty rows visited
    unsigned long long gather_next;             // next query chunk of the FP32 gather
    unsigned long long emit_next;               // next emission index of the persistent photon trace
    double cell_factor;
    double inv_pi_r2;          // 1 / (pi r2) of the current pass, set at pass begin
    int32_t cell_sx;           // x cells per y/z cell (>= 1)
    int32_t pad2;
    int64_t cell_cap;
    unsigned long long photon_cap;   // buffers hold at most this many photons
    unsigned long long hit_cap;      // and this many hit points
    unsigned long long photon_rays;         // photon ray segments traced this pass (one per event)
    unsigned long long eq[MAX_TRACE + 2];   // eye-tree vertices at each depth
    uint32_t hb_lo[3], hb_hi[3];            // hit point bounds (orderable FP32 encodings)
    unsigned long long tile_items;          // tile gather: items queued this pass
    unsigned long long tile_next;           // and the next one to take
    int32_t scene_box;                      // 1: every object is bounded; the grid spans their box
    uint32_t trace_done;                    // photon-trace blocks finished this pass
    double scene_lo[3], scene_hi[3];        // the scene's box (photons and hit points lie on its objects)
};

// number of valid photons / hit points (the counters keep counting past the
// capacity on overflow; readers never go beyond the buffers)
// (a host-supplied count n_fixed >= 0 describes a buffer the host sized; only
// device-counted values are clamped)
__device__ __forceinline__ unsigned long long n_photons(const PassState *st, long long n_fixed) {
    if (n_fixed >= 0) return (unsigned long long)n_fixed;
    unsigned long long n = st->n_stored;
    return n < st->photon_cap ? n : st->photon_cap;
}
__device__ __forceinline__ unsigned long long n_hitpoints(const PassState *st, long long n_fixed) {
    if (n_fixed >= 0) return (unsigned long long)n_fixed;
    unsigned long long n = st->n_hits;
    return n < st->hit_cap ? n : st->hit_cap;
}

// monotone f64 <-> u64 encoding for atomicMin/atomicMax on bounds
__device__ __forceinline__ unsigned long long ord_enc(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double ord_dec(unsigned long long e) {
    unsigned long long b = (e >> 63) ? (e & 0x7fffffffffffffffULL) : ~e;
    return __longlong_as_double((long long)b);
}

// orderable encoding of a float for atomicMin / atomicMax on unsigned words
__host__ __device__ __forceinline__ uint32_t ordf_enc(uint32_t bits) {
    return (bits >> 31) ? ~bits : (bits | 0x80000000u);
}
__device__ __forceinline__ float ordf_dec(uint32_t e) {
    return __uint_as_float((e >> 31) ? (e & 0x7fffffffu) : ~e);
}

// bits 0..9 of v spread to every third bit (Morton interleave)
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// the hit point sort's grid: 2^7 cubic cells per axis over the hit points'
// bounds, keys are Morton codes
constexpr int HIT_MORTON_BITS = 7;
constexpr long long HIT_KEYS = 1LL << (3 * HIT_MORTON_BITS);

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// programmatic dependent launch (sm_90+): wait for the prerequisite grid to
// finish and flush, and let the dependent grid be scheduled
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dependents_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// warp-aggregated append: returns this lane's slot (called by the lanes that append)
__device__ __forceinline__ unsigned long long agg_append(unsigned long long *ctr) {
    unsigned active = __activemask();
    int leader = __ffs(active) - 1;
    unsigned rank = __popc(active & ((1u << lane_id()) - 1u));
    unsigned long long base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(ctr, (unsigned long long)__popc(active));
    base = __shfl_sync(active, base, leader);
    return base + rank;
}

// octahedral unit-vector encoding, 15 bits per axis + 2-bit wavelength
// (Meyer et al., "On floating-point normal vectors", EGSR 2010)
__device__ __forceinline__ uint32_t oct_pack(float x, float y, float z, int wl) {
    float s = fabsf(x) + fabsf(y) + fabsf(z);
    float inv = s > 0.0f ? 1.0f / s : 0.0f;
    float px = x * inv, py = y * inv;
    if (z < 0.0f) {
        float ox = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float oy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = ox; py = oy;
    }
    uint32_t qx = (uint32_t)__float2int_rn((px * 0.5f + 0.5f) * 32767.0f);
    uint32_t qy = (uint32_t)__float2int_rn((py * 0.5f + 0.5f) * 32767.0f);
    qx = min(qx, 32767u); qy = min(qy, 32767u);
    return qx | (qy << 15) | ((uint32_t)wl << 30);
}
// cos(n, d) for the packed direction d.  Decode: p = q * 2/32767 - 1 per
// component, z = 1 - |px| - |py|; below the equator (z < 0) the octahedron's
// fold maps (px, py) to ((1 - |py|) sign px, (1 - |px|) sign py), written here
// as px - copysign(-z, px) (equal in exact arithmetic, no branch).  The
// normalisation is applied to the dot product.
__device__ __forceinline__ V3<float> oct_raw(uint32_t m, float &inv_len) {
    float px = (float)(m & 32767u) * (2.0f / 32767.0f) - 1.0f;
    float py = (float)((m >> 15) & 32767u) * (2.0f / 32767.0f) - 1.0f;
    const float pz = 1.0f - fabsf(px) - fabsf(py);
    const float t = fmaxf(-pz, 0.0f);
    px -= copysignf(t, px);
    py -= copysignf(t, py);
    inv_len = rsqrtf(__fmaf_rn(pz, pz, __fmaf_rn(py, py, px * px)));
    return mk3(px, py, pz);
}
__device__ __forceinline__ float oct_dot(uint32_t m, V3<float> n) {
    float inv;
    const V3<float> p = oct_raw(m, inv);
    return (n.x * p.x + n.y * p.y + n.z * p.z) * inv;
}

// unsorted photon record of the FP64 path (also the parity download format)
struct PhotonD {
    double pos[3];
    double dir[3];
    int32_t emit;
    int8_t level;
    uint8_t wl;
    int16_t pad;
};

template <typename T> struct PhotonBuf;
template <> struct PhotonBuf<double> {
    PhotonD *raw;          // unsorted
    double4 *spos;         // sorted: x, y, z, meta (orig index | wl << 40)
    double4 *sdir;         // sorted: dx, dy, dz, 0
    __device__ __forceinline__ void write(unsigned long long i, const PhotonPath<double> &ph, V3<double> p) const {
        PhotonD r;
        r.pos[0] = p.x; r.pos[1] = p.y; r.pos[2] = p.z;
        r.dir[0] = ph.dir.x; r.dir[1] = ph.dir.y; r.dir[2] = ph.dir.z;
        r.emit = (int32_t)ph.item; r.level = (int8_t)ph.level; r.wl = (uint8_t)ph.wl; r.pad = 0;
        raw[i] = r;
    }
    __device__ __forceinline__ V3<double> raw_pos(unsigned long long i) const { return ld3(raw[i].pos); }
    __device__ __forceinline__ V3<double> raw_pos_wl(unsigned long long i, int &wl) const {
        wl = raw[i].wl;
        return ld3(raw[i].pos);
    }
};
template <> struct PhotonBuf<float> {
    float4 *raw;           // unsorted: x, y, z, oct(dir) | wl
    float4 *sorted;        // sorted copy
    int32_t *sidx;         // optional: original index per sorted slot
    __device__ __forceinline__ void write(unsigned long long i, const PhotonPath<float> &ph, V3<float> p) const {
        raw[i] = make_float4(p.x, p.y, p.z, __uint_as_float(oct_pack(ph.dir.x, ph.dir.y, ph.dir.z, ph.wl)));
    }
    __device__ __forceinline__ V3<float> raw_pos(unsigned long long i) const {
        float4 r = raw[i];
        return mk3(r.x, r.y, r.z);
    }
    __device__ __forceinline__ V3<float> raw_pos_wl(unsigned long long i, int &wl) const {
        const float4 r = raw[i];
        wl = (int)(__float_as_uint(r.w) >> 30);
        return mk3(r.x, r.y, r.z);
    }
};

template <typename T>
struct HitPoint {
    T pos[3];
    T nrm[3];
    T w[3];
    int32_t pixel;
};

// ---------------------------------------------------------------------------
// wavefront queues: two 4-wide vectors per entry (xyz + a 32-bit tag each)
// ---------------------------------------------------------------------------
template <typename T> struct Vec4T;
template <> struct Vec4T<float> { using type = float4; };
template <> struct Vec4T<double> { using type = double4; };
template <typename T> using vec4_t = typename Vec4T<T>::type;

__device__ __forceinline__ float4 mk4(V3<float> v, uint32_t w) { return make_float4(v.x, v.y, v.z, __uint_as_float(w)); }
__device__ __forceinline__ double4 mk4(V3<double> v, uint32_t w) {
    return make_double4(v.x, v.y, v.z, __longlong_as_double((long long)w));
}
__device__ __forceinline__ V3<float> xyz(float4 v) { return mk3(v.x, v.y, v.z); }
__device__ __forceinline__ V3<double> xyz(double4 v) { return mk3(v.x, v.y, v.z); }
__device__ __forceinline__ uint32_t tag(float4 v) { return __float_as_uint(v.w); }
__device__ __forceinline__ uint32_t tag(double4 v) { return (uint32_t)__double_as_longlong(v.w); }

// photon ray queue: a = (pos, emission index), b = (dir, wl | (medium+1) << 8)

// Grid over the photon bounds with cells of c = r/k * (1 + 1/128) in y and z
// (k = cells per radius) and c / sx in x.  The margin keeps |p - q| <= r  =>
// |cell(p) - cell(q)| <= ext (extx in x) under FP32 rounding of the cell
// coordinate (<= 3 ulp of <= 8192 cells per axis).
__device__ __forceinline__ void grid_setup_state(PassState *st, double r2_override) {
    double r2 = r2_override > 0.0 ? r2_override : st->r2;
    double r = sqrt(r2);
    double lo[3], hi[3];
    bool empty = false;
    for (int a = 0; a < 3; a++) {
        lo[a] = ord_dec(st->bb_lo[a]);
        hi[a] = ord_dec(st->bb_hi[a]);
        if (!(lo[a] <= hi[a])) empty = true;
    }
    for (int a = 0; a < 3; a++)
        if (!(hi[a] - lo[a] >= 0.0 && hi[a] - lo[a] < 1e30)) empty = true;
    if (empty) for (int a = 0; a < 3; a++) { lo[a] = 0.0; hi[a] = 0.0; }
    double k = st->cell_factor > 0.0 ? st->cell_factor : 1.0;
    const int sx = st->cell_sx >= 1 ? st->cell_sx : 1;
    // One thread, and FP64 is a narrow, long-latency pipe on this GPU: two
    // divisions, the rest multiplications by the reciprocal (the same
    // product form cell_of uses, so the last cell holds hi exactly).
    double c = r * ((1.0 + 1.0 / 128.0) / k);
    if (!(c > 0.0 && c < 1e30)) c = 1.0;
    double inv = 1.0 / c;
    long long dim[3] = {1, 1, 1};
    for (int it = 0; it < 400; it++) {
        bool ok = true;
        long long tot = 1;
        for (int a = 0; a < 3; a++) {
            double f = floor((hi[a] - lo[a]) * (a == 0 ? inv * sx : inv));
            if (!(f >= 0.0 && f < 8192.0)) { ok = false; dim[a] = 8193; }
            else dim[a] = (long long)f + 1;
            tot *= dim[a];
        }
        if (ok && tot <= st->cell_cap) break;
        c *= 1.25;
        inv = 1.0 / c;
        if (it == 399) { dim[0] = dim[1] = dim[2] = 1; c = 1e30; inv = 1e-30; }
    }
    GridParams g;
    for (int a = 0; a < 3; a++) {
        g.org[a] = lo[a];
        g.orgf[a] = (float)lo[a];
        g.dim[a] = (int32_t)dim[a];
    }
    const double invx = inv * sx;
    g.cell = c;
    g.inv = inv;
    g.invf = (float)inv;
    g.invx = invx;
    g.invxf = (float)invx;
    double ef = ceil(r * inv + 3e-3);
    int ext = ef >= 1.0 && ef <= 8.0 ? (int)ef : (ef > 8.0 ? 8 : 1);
    g.ext = ext < 1 ? 1 : (ext > 8 ? 8 : ext);
    double efx = ceil(r * invx + 3e-3);
    g.extx = efx >= 1.0 && efx <= 64.0 ? (int)efx : (efx > 64.0 ? 64 : 1);
    g.ncell = dim[0] * dim[1] * dim[2];
    g.nkeys = g.ncell;
    g.r2f = (float)r2;
    g.r2_lo = __double2float_rd(r2 * (1.0 - 1e-6));
    g.r2_hi = __double2float_ru(r2 * (1.0 + 1e-6));
    g.cellf = (float)c;
    st->grid = g;
}

// Scene tables of a box scene (no hierarchy) copied to shared memory by each
// eye-level block: a level after the first has few vertices per SM, and a
// vertex's intersection is then a chain of object loads from L2 (the table
// is not yet in this SM's L1), one round trip per object.  Larger tables
// stay in global memory.
constexpr int EYE_SMEM_OBJS = 32, EYE_SMEM_MATS = 32;

template <typename T, bool B>
__device__ __forceinline__ SceneView<T, B> stage_scene(const SceneView<T, B> &sc) {
    SceneView<T, B> v = sc;
    if constexpr (!B) {
        constexpr int OW = (int)(sizeof(DObject<T>) / 4), MW = (int)(sizeof(DMaterial<T>) / 4);
        static_assert(sizeof(DMaterial<T>) % 4 == 0, "materials copy as 32-bit words");
        __shared__ __align__(16) uint32_t s_obj[EYE_SMEM_OBJS * OW];
        __shared__ __align__(16) uint32_t s_mat[EYE_SMEM_MATS * MW];
        if (sc.n_objs <= EYE_SMEM_OBJS && sc.n_mats <= EYE_SMEM_MATS) {   // uniform over the block
            const uint32_t *go = reinterpret_cast<const uint32_t *>(sc.objs);
            const uint32_t *gm = reinterpret_cast<const uint32_t *>(sc.mats);
            for (int k = threadIdx.x; k < sc.n_objs * OW; k += blockDim.x) s_obj[k] = __ldg(go + k);
            for (int k = threadIdx.x; k < sc.n_mats * MW; k += blockDim.x) s_mat[k] = __ldg(gm + k);
            __syncthreads();
            v.objs = reinterpret_cast<const DObject<T> *>(s_obj);
            v.mats = reinterpret_cast<const DMaterial<T> *>(s_mat);
        }
    }
    return v;
}

// The persistent photon trace runs in blocks of TRACE_THREADS; TraceBlocks
// is the most that stay resident per SM: 16 in FP32 (64 registers, no
// spills), 8 in FP64.  Box scenes in FP32 launch TRACE_BLOCKS_BESIDE_EYE
// per SM instead, leaving registers for one block of the eye levels (128
// threads at 96 registers): 13 x 64 x 64 + 128 x 96 = 65,536, the SM's
// register file.  Small blocks keep that room small: six of 128 threads
// leave more, and measured 1 % slower on the glass box; sixteen of 64 leave
// none, and the deeper eye levels then wait for the trace to end.
constexpr int TRACE_THREADS = 64;
template <typename T> struct TraceBlocks { static constexpr int value = 8; };
template <> struct TraceBlocks<float> { static constexpr int value = 16; };
constexpr int TRACE_BLOCKS_BESIDE_EYE = 13;

// Persistent photon tracing: one launch per pass (measured faster than an
// emission kernel plus MAX_TRACE bounce kernels with ray queues between them,
// on the glass box and on the 1.3M-triangle mesh).  Each lane
// carries one photon through one event per iteration; a lane whose photon
// ended takes the next emission index (one atomic per warp for all its idle
// lanes), so lanes stay busy until the emission list runs out, and no ray
// goes through memory between bounces.  Random streams are keyed by
// (emission index, pass, level) as in the wavefront form, so the stored
// photons are the same set (their order in the buffer differs).
template <typename T, bool B>
__global__ void __launch_bounds__(TRACE_THREADS, TraceBlocks<T>::value)
    k_trace(SceneView<T, B> sc, EmitPlan plan, uint64_t seed, PassState *st, int uc, PhotonBuf<T> photons) {
    const uint32_t pass = (uint32_t)st->pass;
    const unsigned long long n_emit = (unsigned long long)plan.first[plan.n_lights];
    const unsigned long long pcap = st->photon_cap;
    const unsigned lane = lane_id();
    PhotonPath<T> ph;
    ph.level = 0;
    bool active = false, exhausted = false;
    unsigned rays = 0;
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !active) & (exhausted ? 0u : 0xffffffffu);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(&st->emit_next, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + __popc(need) >= n_emit) exhausted = true;
            if (!active) {
                const unsigned long long i = base + __popc(need & ((1u << lane) - 1u));
                if (i < n_emit) {
                    int li = 0;
                    while (li < plan.n_lights - 1 && (int64_t)i >= plan.first[li + 1]) li++;
                    Rng rg;
                    rg.init<T>(seed, (uint32_t)i, pass, TAG_EMIT);
                    generate_photon(sc.lights[li], rg, ph);
                    ph.item = (uint32_t)i;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) {
            rays++;
            const PhotonPath<T> cur = ph;
            bool store;
            V3<T> spos;
            const bool alive = photon_event(sc, seed, pass, uc != 0, ph, store, spos);
            if (store) {
                unsigned long long slot = agg_append(&st->n_stored);
                if (slot < pcap) photons.write(slot, cur, spos);
                else atomicOr(&st->overflow, 1u);
            }
            ph.level = cur.level + 1;
            active = alive && ph.level < MAX_TRACE;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rays += __shfl_xor_sync(0xffffffffu, rays, o);
    if (lane == 0 && rays) atomicAdd(&st->photon_rays, (unsigned long long)rays);
    // FP32 box scenes: the pass's grid spans the scene's box, which the
    // photons do not change, so the first block to finish sets it up here
    // (after its loop, out of the loop's register budget, while the other
    // blocks still trace) and the map build follows the trace with no
    // set-up kernel between them
    if constexpr (sizeof(T) == 4)
        if (st->scene_box) {   // uniform over the block
            __syncthreads();
            if (threadIdx.x == 0 && atomicAdd(&st->trace_done, 1u) == 0u) grid_setup_state(st, -1.0);
        }
    grid_dependents_launch();   // the map build may be scheduled once every block is here
}

// bounds of n photons (block reduction, then one atomic per block and axis)
template <typename T>
__global__ void __launch_bounds__(256) k_bbox(PhotonBuf<T> buf, PassState *st, long long n_fixed) {
    grid_dependency_wait();
    unsigned long long n = n_photons(st, n_fixed);
    // reduced in the photons' own precision; converted once per block
    T lo[3] = {T(1e30), T(1e30), T(1e30)}, hi[3] = {T(-1e30), T(-1e30), T(-1e30)};
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        V3<T> p = buf.raw_pos(i);
        T v[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (v[a] > T(-1e30) && v[a] < T(1e30)) {   // finite and bounded (false for NaN)
                lo[a] = v[a] < lo[a] ? v[a] : lo[a];
                hi[a] = v[a] > hi[a] ? v[a] : hi[a];
            }
        }
    }
    __shared__ T slo[3][8], shi[3][8];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            T ol = __shfl_xor_sync(0xffffffffu, lo[a], o), oh = __shfl_xor_sync(0xffffffffu, hi[a], o);
            lo[a] = ol < lo[a] ? ol : lo[a];
            hi[a] = oh > hi[a] ? oh : hi[a];
        }
        if (lane_id() == 0) { slo[a][threadIdx.x >> 5] = lo[a]; shi[a][threadIdx.x >> 5] = hi[a]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int a = threadIdx.x;
        T l = slo[a][0], h = shi[a][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            l = slo[a][w] < l ? slo[a][w] : l;
            h = shi[a][w] > h ? shi[a][w] : h;
        }
        if (l <= h) {
            atomicMin(&st->bb_lo[a], ord_enc((double)l));
            atomicMax(&st->bb_hi[a], ord_enc((double)h));
        }
    }
    grid_dependents_launch();
}

// cell coordinate, clamped to the grid
template <typename T> struct CellMath;
template <> struct CellMath<double> {
    __device__ static __forceinline__ int coord(const GridParams &g, double p, int a) {
        double f = floor((p - g.org[a]) * (a == 0 ? g.invx : g.inv));
        f = fmin(fmax(f, 0.0), (double)(g.dim[a] - 1));
        return (int)f;
    }
};
template <> struct CellMath<float> {
    __device__ static __forceinline__ int coord(const GridParams &g, float p, int a) {
        float f = floorf((p - g.orgf[a]) * (a == 0 ? g.invxf : g.invf));
        f = fminf(fmaxf(f, 0.0f), (float)(g.dim[a] - 1));
        return (int)f;
    }
};

template <typename T>
__device__ __forceinline__ uint32_t cell_of(const GridParams &g, V3<T> p) {
    int cx = CellMath<T>::coord(g, p.x, 0), cy = CellMath<T>::coord(g, p.y, 1), cz = CellMath<T>::coord(g, p.z, 2);
    return (uint32_t)((cz * g.dim[1] + cy) * g.dim[0] + cx);
}

template <typename T>
__global__ void __launch_bounds__(256) k_cell_hist(PhotonBuf<T> buf, PassState *st, long long n_fixed,
                                                   uint32_t *count, uint2 *keyrank) {
    grid_dependency_wait();
    unsigned long long n = n_photons(st, n_fixed);
    const GridParams g = st->grid;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t c = cell_of(g, buf.raw_pos(i));
        const uint32_t r = atomicAdd(&count[c], 1u);
        keyrank[i] = make_uint2(c, r);
    }
    grid_dependents_launch();
}

template <typename T> __global__ void k_scatter(PhotonBuf<T> buf, PassState *st, long long n_fixed,
                                                const uint32_t *start, const uint2 *keyrank);

#if defined(PPM_BUILD_F64)
template <>
__global__ void __launch_bounds__(256) k_scatter<double>(PhotonBuf<double> buf, PassState *st, long long n_fixed,
                                                         const uint32_t *start, const uint2 *keyrank) {
    grid_dependency_wait();
    unsigned long long n = n_photons(st, n_fixed);
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint2 kr = keyrank[i];
        uint32_t dst = start[kr.x] + kr.y;
        const PhotonD r = buf.raw[i];
        unsigned long long meta = (unsigned long long)i | ((unsigned long long)r.wl << 40);
        buf.spos[dst] = make_double4(r.pos[0], r.pos[1], r.pos[2], __longlong_as_double((long long)meta));
        buf.sdir[dst] = make_double4(r.dir[0], r.dir[1], r.dir[2], 0.0);
    }
    grid_dependents_launch();
}

#endif

#if defined(PPM_BUILD_F32)
template <>
__global__ void __launch_bounds__(256) k_scatter<float>(PhotonBuf<float> buf, PassState *st, long long n_fixed,
                                                        const uint32_t *start, const uint2 *keyrank) {
    grid_dependency_wait();
    unsigned long long n = n_photons(st, n_fixed);
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint2 kr = keyrank[i];
        uint32_t dst = start[kr.x] + kr.y;
        buf.sorted[dst] = buf.raw[i];
        if (buf.sidx) buf.sidx[dst] = (int32_t)i;
    }
    grid_dependents_launch();
}

#endif

// ---------------------------------------------------------------------------
// eye pass: camera rays (camera.rs:58-75) and the eye tree (tracer.rs:129-177)
// evaluated level by level.  Every vertex carries the product of the bsdf
// weights on its path (the bsdf is linear in di, si, ti, surface.rs:135-206),
// adds throughput x (emittance/2pi + c_di x direct light) to its pixel and
// appends a hit point with weight throughput x c_di for the photon estimate;
// its reflected and refracted children go to the next level's queue.
// Queue entry: a = (pos, pixel), b = (dir, node | (medium+1) << 16), c = (w, 0).
// ---------------------------------------------------------------------------
template <typename T>
struct EyeQueue {
    vec4_t<T> *a, *b, *c;
};

// Pixel output of the eye pass.  FP64 path: the pass image itself.  FP32
// path: the per-pass direct-light buffer (FP32), and level 0 also clears the
// per-pass gathered-flux buffer of its pixel.
template <typename T> struct EyeOut;
template <> struct EyeOut<double> {
    double *img;
    __device__ __forceinline__ void set(uint32_t p, V3<double> v) const {
        img[3 * (size_t)p] = v.x; img[3 * (size_t)p + 1] = v.y; img[3 * (size_t)p + 2] = v.z;
    }
    __device__ __forceinline__ void add(uint32_t p, V3<double> v) const {
        atomicAdd(img + 3 * (size_t)p, v.x); atomicAdd(img + 3 * (size_t)p + 1, v.y); atomicAdd(img + 3 * (size_t)p + 2, v.z);
    }
};
template <> struct EyeOut<float> {
    float *direct;
    float *gathered;
    __device__ __forceinline__ void set(uint32_t p, V3<float> v) const {
        direct[3 * (size_t)p] = v.x; direct[3 * (size_t)p + 1] = v.y; direct[3 * (size_t)p + 2] = v.z;
        gathered[3 * (size_t)p] = 0.f; gathered[3 * (size_t)p + 1] = 0.f; gathered[3 * (size_t)p + 2] = 0.f;
    }
    __device__ __forceinline__ void add(uint32_t p, V3<float> v) const {
        atomicAdd(direct + 3 * (size_t)p, v.x); atomicAdd(direct + 3 * (size_t)p + 1, v.y);
        atomicAdd(direct + 3 * (size_t)p + 2, v.z);
    }
};

// Camera rays are launched in tiles of EYE_TILE_W x EYE_TILE_H pixels, one
// tile per warp (tiles row-major over the image, pixels row-major inside a
// tile), so that the hit points a warp appends are a compact patch of the
// scene: the render gather takes hit points 32 at a time and walks the
// photons around all of them once.  Slots of tiles that overhang the image
// edge have no pixel.  The random streams are keyed by pixel, so the order
// changes no result.
constexpr int EYE_TILE_W = 4, EYE_TILE_H = 8;
static_assert(EYE_TILE_W * EYE_TILE_H == 32, "one tile per warp");
__host__ __device__ __forceinline__ long long eye_tiles_x(int xreso) { return (xreso + EYE_TILE_W - 1) / EYE_TILE_W; }
__host__ __device__ __forceinline__ long long eye_slots(int xreso, int yreso) {
    return eye_tiles_x(xreso) * ((yreso + EYE_TILE_H - 1) / EYE_TILE_H) * 32;
}

// CLASSIC: trace_ray_classic (tracer.rs:221-259) instead of trace_ray:
// direct light of every light plus the camera's ambient, no hit points, the
// exact mirror direction, refraction about the normal with the child's
// medium by the side the refracted ray leaves on, and the bsdf at cos1.
// One vertex of the eye tree: slot i of level 0 (a camera ray) or entry i
// of the level's queue.
template <typename T, bool B, bool CLASSIC = false>
__device__ __forceinline__ void eye_vertex(const SceneView<T, B> &sc, const DCamera<T> &cam, uint64_t seed,
                                           PassState *st, int uc, int level, EyeQueue<T> in, EyeQueue<T> out,
                                           unsigned long long qcap, HitPoint<T> *hits, EyeOut<T> pix,
                                           unsigned long long i, uint32_t pass, unsigned long long hit_cap,
                                           long long ntx) {
    const T air[3] = {T(1), T(1), T(1)};
    {
        V3<T> rp, rd, w;
        uint32_t p, node;
        int medium;
        if (level == 0) {
            const uint32_t tile = (uint32_t)(i >> 5), k = (uint32_t)(i & 31);
            const uint32_t px = (tile % (uint32_t)ntx) * EYE_TILE_W + k % EYE_TILE_W;
            const uint32_t py = (tile / (uint32_t)ntx) * EYE_TILE_H + k / EYE_TILE_W;
            if (px >= (uint32_t)cam.xreso || py >= (uint32_t)cam.yreso) return;
            p = py * (uint32_t)cam.xreso + px;
            const T y = (T)py, x = (T)px;
            Rng rg;
            rg.init<T>(seed, p, pass, TAG_CAMERA);
            V3<T> blur = mk3(T(0), T(0), T(0));
            if (cam.blur) {
                T r1 = gen_range<T>(rg, T(-0.5), T(0.5));
                T r2 = gen_range<T>(rg, T(-0.5), T(0.5));
                blur = r1 * ld3(cam.eex) + r2 * ld3(cam.eey);
            }
            T r3 = T(0), r4 = T(0);
            if (cam.jitter_aa) {
                r3 = gen_range<T>(rg, T(-0.5), T(0.5));
                r4 = gen_range<T>(rg, T(-0.5), T(0.5));
            }
            rp = ld3(cam.eye) + blur;
            V3<T> ed = ((ld3(cam.origin) + (x + r3) * ld3(cam.esx)) + (y + r4) * ld3(cam.esy)) - blur;
            rd = ed;
            normalize(ed, rd);
            w = mk3(T(1), T(1), T(1));
            node = 1u;
            medium = -1;
        } else {
            const vec4_t<T> a = in.a[i], b = in.b[i], c = in.c[i];
            rp = xyz(a);
            p = tag(a);
            rd = xyz(b);
            node = tag(b) & 0xffffu;
            medium = (int)(tag(b) >> 16) - 1;
            w = xyz(c);
        }
        V3<T> acc = mk3(T(0), T(0), T(0));
        Isect<T> is;
        if (intersect(sc, rp, rd, is)) {
            const int mid = sc.objs[is.obj].mat;
            const DMaterial<T> &mate = sc.mats[mid];
            acc = hmul(w, ld3(mate.emit)) * Cst<T>::sr_half();
            Coef<T> cf;
            V3<T> rdir = is.n, td = is.n;
            T cos1;
            bool has_t = false;
            const bool diffuse_only = mate.surface == SF_SIMPLE && mate.scatter == T(1);
            if (diffuse_only) {
                // Simple surface with diffuseness 1: no reflected child, the
                // refracted child has weight 0 and c_di does not depend on cos
                cf = bsdf_coef(mate, T(0));
                cos1 = T(0);
            } else {
                T cos2;
                V3<T> rdir0 = specular_reflection(is.n, rd, cos1);
                T eta = relative_ior_average(ior_of(sc, medium, air), mate.ior);
                if constexpr (CLASSIC) {
                    rdir = rdir0;
                    has_t = specular_refraction(is.n, rd, eta, td, cos2);
                    cf = bsdf_coef(mate, cos1);
                } else {
                    Rng rv;
                    rv.init<T>(seed, p, pass, TAG_EYE | node);
                    rdir = reflection_glossy(rv, is.n, rdir0, sf_power_glossy(mate));
                    V3<T> hvec = is.n;
                    if (!normalize(rdir - rd, hvec)) hvec = is.n;
                    has_t = specular_refraction(hvec, rd, eta, td, cos2);
                    T cos = cos1 < cos2 ? cos1 : cos2;
                    cf = bsdf_coef(mate, cos);
                }
            }
            const V3<T> W = hmul(w, cf.di);
            if (CLASSIC && any_nz(W)) {
                V3<T> di = ld3(cam.ambient);
                for (int l = 0; l < sc.n_lights; l++) di = di + radiance_from_light(sc, is.pos, is.n, sc.lights[l]);
                acc = acc + hmul(W, di);
            } else if (any_nz(W)) {
                if (uc) {
                    V3<T> di = mk3(T(0), T(0), T(0));
                    for (int l = 0; l < sc.n_lights; l++) di = di + radiance_from_light(sc, is.pos, is.n, sc.lights[l]);
                    acc = acc + hmul(W, di);
                }
                unsigned long long slot = agg_append(&st->n_hits);
                if (slot < hit_cap) {
                    HitPoint<T> h;
                    h.pos[0] = is.pos.x; h.pos[1] = is.pos.y; h.pos[2] = is.pos.z;
                    h.nrm[0] = is.n.x; h.nrm[1] = is.n.y; h.nrm[2] = is.n.z;
                    h.w[0] = W.x; h.w[1] = W.y; h.w[2] = W.z;
                    h.pixel = (int32_t)p;
                    hits[slot] = h;
                } else {
                    atomicOr(&st->overflow, 2u);
                }
            }
            if (!diffuse_only && level + 1 < MAX_TRACE) {
                const V3<T> ws = hmul(w, cf.si);
                if (sf_reflect(mate, cos1) && any_nz(ws)) {
                    unsigned long long o = agg_append(&st->eq[level + 1]);
                    if (o < qcap) {
                        out.a[o] = mk4(is.pos, p);
                        out.b[o] = mk4(rdir, (2u * node) | ((uint32_t)(medium + 1) << 16));
                        out.c[o] = mk4(ws, 0u);
                    } else {
                        atomicOr(&st->overflow, 4u);
                    }
                }
                const V3<T> wt = hmul(w, cf.ti);
                if (has_t && sf_refract(mate, cos1) && any_nz(wt)) {
                    unsigned long long o = agg_append(&st->eq[level + 1]);
                    if (o < qcap) {
                        out.a[o] = mk4(is.pos, p);
                        const int m2 = CLASSIC ? (dot(td, is.n) < T(0) ? mid : -1) : (is.in ? mid : -1);
                        out.b[o] = mk4(td, (2u * node + 1u) | ((uint32_t)(m2 + 1) << 16));
                        out.c[o] = mk4(wt, 0u);
                    } else {
                        atomicOr(&st->overflow, 4u);
                    }
                }
            }
        }
        if (level == 0) pix.set(p, acc);
        else if (any_nz(acc)) pix.add(p, acc);
    }
}

template <typename T, bool B, bool CLASSIC = false>
__device__ __forceinline__ void eye_level(const SceneView<T, B> &gsc, const DCamera<T> &cam, uint64_t seed,
                                          PassState *st, int uc, int level, EyeQueue<T> in, EyeQueue<T> out,
                                          unsigned long long qcap, HitPoint<T> *hits, EyeOut<T> pix) {
    // the scene's tables do not change within a pass: staged before the wait
    const SceneView<T, B> sc = stage_scene(gsc);
    // Levels after 0 are programmatic dependents of the level before: their
    // blocks may be scheduled before it ends and wait here until it has
    // finished and its queue appends are visible (a no-op for a plain launch)
    grid_dependency_wait();
    const uint32_t pass = (uint32_t)st->pass;
    const unsigned long long hit_cap = st->hit_cap;
    const long long ntx = eye_tiles_x(cam.xreso);
    unsigned long long n = level == 0 ? (unsigned long long)eye_slots(cam.xreso, cam.yreso) : st->eq[level];
    if (level > 0 && n > qcap) n = qcap;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        eye_vertex<T, B, CLASSIC>(sc, cam, seed, st, uc, level, in, out, qcap, hits, pix, i, pass, hit_cap, ntx);
    // this block's work is done: the next level may be scheduled once every
    // block has said so, i.e. once every block of this level has been
    // scheduled, so its waiting blocks can never hold slots this level needs
    grid_dependents_launch();
}

// Two entry points over the same body: without a hierarchy five blocks per
// SM (96 registers in FP32: one block fits beside the photon trace's
// TRACE_BLOCKS_BESIDE_EYE); with one, a cap of 128 registers, under which
// the traversal stack does not spill.
template <typename T, bool CLASSIC>
__global__ void __launch_bounds__(128, 5) k_eye_level(SceneView<T, false> sc, DCamera<T> cam, uint64_t seed,
                                                      PassState *st, int uc, int level, EyeQueue<T> in,
                                                      EyeQueue<T> out, unsigned long long qcap, HitPoint<T> *hits,
                                                      EyeOut<T> pix) {
    eye_level<T, false, CLASSIC>(sc, cam, seed, st, uc, level, in, out, qcap, hits, pix);
}
template <typename T, bool CLASSIC>
__global__ void __maxnreg__(128) k_eye_level_bvh(SceneView<T, true> sc, DCamera<T> cam, uint64_t seed, PassState *st,
                                                 int uc, int level, EyeQueue<T> in, EyeQueue<T> out,
                                                 unsigned long long qcap, HitPoint<T> *hits, EyeOut<T> pix) {
    eye_level<T, true, CLASSIC>(sc, cam, seed, st, uc, level, in, out, qcap, hits, pix);
}

// ---------------------------------------------------------------------------
// candidate enumeration: the (2e+1)^2 x-rows of cells around a query (each
// row spans 2e+1 cells, contiguous in the sorted map).  Lane j holds row j
// (rows in chunks of 32); the warp walks the non-empty rows in order and its
// lanes stride through each row, so a candidate costs an increment, not a
// search.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void query_cells(const GridParams &g, V3<T> q, int ext, int extx, int c[3], int lo[3],
                                            int hi[3]) {
    c[0] = CellMath<T>::coord(g, q.x, 0);
    c[1] = CellMath<T>::coord(g, q.y, 1);
    c[2] = CellMath<T>::coord(g, q.z, 2);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int e = a == 0 ? extx : ext;
        lo[a] = max(c[a] - e, 0);
        hi[a] = min(c[a] + e, g.dim[a] - 1);
    }
}

struct RowSet {
    uint32_t begin, len;   // this lane's row (culled x-range)
    unsigned nonempty;     // ballot of rows with len > 0
};

// Row culling: the row (yy, zz) can hold a photon within r of q only where
// the sphere reaches its y/z slab; its x-range shrinks to the sphere's chord
// there.  The slab bounds are widened and the chord lengthened by margins
// that exceed the rounding of the cell coordinates (<= 3 ulp of <= 8192
// cells), so the culled set still contains every photon within r; the exact
// predicate then decides membership.
template <typename T> struct RowCull;
template <> struct RowCull<float> {
    __device__ static __forceinline__ bool range(const GridParams &g, V3<float> q, float r2, int yy, int zz,
                                                 int lo_x, int hi_x, int &x0, int &x1) {
        const float c = g.cellf, m = 4e-3f * c;
        const float ylo = g.orgf[1] + (float)yy * c, zlo = g.orgf[2] + (float)zz * c;
        const float dy = fmaxf(0.0f, fmaxf(ylo - q.y, q.y - (ylo + c)) - m);
        const float dz = fmaxf(0.0f, fmaxf(zlo - q.z, q.z - (zlo + c)) - m);
        const float rem = r2 * 1.00002f - dy * dy - dz * dz;
        if (rem < 0.0f) return false;
        const float rx = sqrtf(rem) * 1.00001f;
        const float fx0 = floorf((q.x - rx - g.orgf[0]) * g.invxf - 4e-3f);
        const float fx1 = floorf((q.x + rx - g.orgf[0]) * g.invxf + 4e-3f);
        x0 = max(lo_x, (int)fmaxf(fx0, -1.0f));
        x1 = min(hi_x, (int)fminf(fx1, (float)g.dim[0]));
        return x0 <= x1;
    }
};
template <> struct RowCull<double> {
    __device__ static __forceinline__ bool range(const GridParams &g, V3<double> q, double r2, int yy, int zz,
                                                 int lo_x, int hi_x, int &x0, int &x1) {
        const double c = g.cell, m = 1e-6 * c;
        const double ylo = g.org[1] + (double)yy * c, zlo = g.org[2] + (double)zz * c;
        const double dy = fmax(0.0, fmax(ylo - q.y, q.y - (ylo + c)) - m);
        const double dz = fmax(0.0, fmax(zlo - q.z, q.z - (zlo + c)) - m);
        const double rem = r2 * (1.0 + 1e-12) - dy * dy - dz * dz;
        if (rem < 0.0) return false;
        const double rx = sqrt(rem) * (1.0 + 1e-12);
        const double fx0 = floor((q.x - rx - g.org[0]) * g.invx - 1e-6);
        const double fx1 = floor((q.x + rx - g.org[0]) * g.invx + 1e-6);
        x0 = max(lo_x, (int)fmax(fx0, -1.0));
        x1 = min(hi_x, (int)fmin(fx1, (double)g.dim[0]));
        return x0 <= x1;
    }
};

template <typename T>
__device__ __forceinline__ RowSet make_rows(const GridParams &g, const uint32_t *start, V3<T> q, T r2, const int lo[3],
                                            const int hi[3], int row0) {
    const int ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const int nrows = ny * nz;
    int row = row0 + (int)lane_id();
    RowSet rs;
    rs.begin = 0;
    rs.len = 0;
    int x0, x1;
    if (row < nrows) {
        // row / ny without an integer division: (row + 1/2) / ny is at least
        // 1/(2 ny) >= 1/34 from an integer (ny = 2 ext + 1 <= 17) and, with
        // row < 2^10, __fdividef's error is below 2^-10, so truncation is exact
        int zi = __float2int_rz(__fdividef((float)row + 0.5f, (float)ny));
        int yy = lo[1] + (row - zi * ny), zz = lo[2] + zi;
        if (RowCull<T>::range(g, q, r2, yy, zz, lo[0], hi[0], x0, x1)) {
            int base = (zz * g.dim[1] + yy) * g.dim[0];
            rs.begin = start[base + x0];
            rs.len = start[base + x1 + 1] - rs.begin;
        }
    }
    rs.nonempty = __ballot_sync(0xffffffffu, rs.len > 0);
    return rs;
}

// Packed rows: a group's non-empty rows laid end to end, walked in windows
// of 32 positions, so that a row of 9 candidates and the next of 40 fill
// two windows rather than three mostly idle ones.  Position p of the
// concatenation is in the row whose start is the last one at or before p:
// a window ORs the bits (start - window base) of the starts that fall in
// it (one reduction), and lane i counts the bits at or below i.  Lane k of
// the warp holds, for the k-th non-empty row, the map slot of its first
// candidate minus its start, so the slot of position p is one shuffle and
// one add away.  No search, no shared memory.
struct PackedRows {
    uint32_t total;   // candidates in the group's rows
    uint32_t first;   // this lane's row's start in the concatenation (0x80000000: empty row)
    uint32_t delta;   // lane k: k-th non-empty row's first slot minus its start
};

__device__ __forceinline__ unsigned lanemask_le() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
    return m;
}

// position of the k-th (from 0) set bit of m; any value in [0, 31] when m
// has k or fewer set bits
__device__ __forceinline__ int kth_set_bit(unsigned m, int k) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) {
        const int c = __popc(m & ((1u << w) - 1u));
        if (k >= c) {
            k -= c;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

// lane i holds row i of the group (first slot rbeg, rlen candidates);
// nonempty is the ballot of rlen > 0
__device__ __forceinline__ PackedRows pack_rows(uint32_t rbeg, uint32_t rlen, unsigned nonempty) {
    const unsigned lane = lane_id();
    uint32_t incl = rlen;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += t;
    }
    PackedRows pr;
    pr.total = __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t s = incl - rlen;
    pr.first = rlen > 0u ? s : 0x80000000u;
    pr.delta = __shfl_sync(0xffffffffu, rbeg - s, kth_set_bit(nonempty, (int)lane));
    return pr;
}

// map slot of position wb + lane (the window at wb; windows in increasing
// order, kbase = -1 before the first); valid = the position holds a
// candidate.  Past the end the slot is the last candidate's, so loads stay
// in bounds.  All lanes must call it.
__device__ __forceinline__ uint32_t packed_slot(const PackedRows &pr, uint32_t wb, unsigned le, int &kbase,
                                                bool &valid) {
    unsigned bit;
    // PTX clamps shift counts above 31: starts outside the window give 0
    asm("shl.b32 %0, %1, %2;" : "=r"(bit) : "r"(1u), "r"(pr.first - wb));
    const unsigned m = __reduce_or_sync(0xffffffffu, bit);
    const int k = kbase + __popc(m & le);
    kbase += __popc(m);
    const uint32_t p = wb + lane_id();
    valid = p < pr.total;
    return min(p, pr.total - 1u) + __shfl_sync(0xffffffffu, pr.delta, k);
}

// calls f(photon_index, valid) for every candidate of the query, lanes in
// parallel; all lanes of the warp must enter (warp-uniform query)
template <typename T, typename F>
__device__ __forceinline__ void for_each_candidate(const GridParams &g, const uint32_t *start, V3<T> q, T r2,
                                                   const int lo[3], const int hi[3], F &&f) {
    const int nrows = (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    for (int row0 = 0; row0 < nrows; row0 += 32) {
        RowSet rs = make_rows(g, start, q, r2, lo, hi, row0);
        unsigned m = rs.nonempty;
        while (m) {
            int r = __ffs(m) - 1;
            m &= m - 1;
            uint32_t b = __shfl_sync(0xffffffffu, rs.begin, r);
            uint32_t n = __shfl_sync(0xffffffffu, rs.len, r);
            // warp-uniform trip count: every lane runs every iteration (lanes
            // past the row end with valid = false), so warp-collective code
            // inside f is reached by the whole warp at the same point
            for (uint32_t base = 0; base < n; base += 32) {
                uint32_t o = base + lane_id();
                f(o < n ? b + o : 0u, o < n);
            }
        }
    }
}

// The render row walk: the group's rows packed end to end (pack_rows), two
// windows per step (both candidates loaded before either is used), handed
// to one call, use(two, p0, valid0, slot0, p1, valid1, slot1), so that
// their radius tests and direction decodes form two independent
// instruction chains in one block (one branch per step instead of two).  A
// step over the last 32 or fewer positions passes two = std::false_type
// and no second photon, so that the body compiled for it does one
// candidate's work.  Every lane makes every call, so use() may hold warp
// votes.  The slots (map positions) are used by the parity export only;
// the production body ignores them.
template <typename U>
__device__ __forceinline__ void for_each_candidate_two(const GridParams &g, const uint32_t *start, V3<float> q,
                                                       float r2, const int lo[3], const int hi[3],
                                                       const float4 *smap, U &&use) {
    const int nrows = (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    const unsigned le = lanemask_le();
    for (int row0 = 0; row0 < nrows; row0 += 32) {
        const RowSet rs = make_rows(g, start, q, r2, lo, hi, row0);
        if (rs.nonempty == 0u) continue;
        const PackedRows pr = pack_rows(rs.begin, rs.len, rs.nonempty);
        int kbase = -1;
        for (uint32_t wb = 0; wb < pr.total; wb += 64) {
            bool v0, v1;
            const uint32_t i0 = packed_slot(pr, wb, le, kbase, v0);
            const float4 p0 = __ldg(&smap[i0]);
            if (wb + 32 < pr.total) {
                const uint32_t i1 = packed_slot(pr, wb + 32, le, kbase, v1);
                const float4 p1 = __ldg(&smap[i1]);
                use(std::true_type{}, p0, v0, i0, p1, v1, i1);
            } else {
                use(std::false_type{}, p0, v0, i0, p0, false, i0);   // the last 32 or fewer
            }
        }
    }
}

__device__ __forceinline__ double filter_wt(int pfilter, double d, double r2) {
    if (pfilter == PF_CONE) {   // tracer.rs:201-204
        double d2 = sqrt(d / r2) / 1.1;
        return d2 > 1.0 ? 0.0 : (1.0 - d2) / (1.0 - 2.0 / (3.0 * 1.1));
    }
    if (pfilter == PF_GAUSS) {  // tracer.rs:213-216
        double e_r = 1.0 - pm_exp(-1.953 * d / (r2 * 2.0));
        double eb = 1.0 - 0.14184788965323;
        return e_r > eb ? 0.0 : 0.918 * (1.0 - e_r / eb) + 0.5;
    }
    return 1.0;
}

// squared_euclidean(query, point) as the kdtree crate sums it
__device__ __forceinline__ double sq_euclid(double qx, double qy, double qz, double px, double py, double pz) {
    double dx = qx - px, dy = qy - py, dz = qz - pz;
    double s = 0.0;
    s = __dadd_rn(s, __dmul_rn(dx, dx));
    s = __dadd_rn(s, __dmul_rn(dy, dy));
    s = __dadd_rn(s, __dmul_rn(dz, dz));
    return s;
}

// ---------------------------------------------------------------------------
// FP64 gather over the sorted double map.  mode 0: render (atomicAdd
// W * estimate into pass_img); mode 1: per-query estimate into out_rgb.
// ---------------------------------------------------------------------------
struct GatherOutD {
    double *pass_img;
    double *out_rgb;
    unsigned long long *count;  // optional candidate / in-radius counters
};

#if defined(PPM_BUILD_F64)
__global__ void __launch_bounds__(256) k_gather_d(const HitPoint<double> *hits, PassState *st, long long n_fixed,
                                                  const double4 *spos, const double4 *sdir, const uint32_t *start,
                                                  double pw, int pfilter, int mode, GatherOutD out) {
    const unsigned long long nq = n_hitpoints(st, n_fixed);
    const GridParams g = st->grid;
    const double r2 = st->r2;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long qi = warp; qi < nq; qi += nwarps) {
        const HitPoint<double> h = hits[qi];
        V3<double> q = ld3(h.pos), n = ld3(h.nrm);
        int c[3], lo[3], hi[3];
        query_cells(g, q, g.ext, g.extx, c, lo, hi);
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for_each_candidate(g, start, q, r2, lo, hi, [&](uint32_t idx, bool valid) {
            if (!valid) return;
            double4 pp = spos[idx];
            double d = sq_euclid(q.x, q.y, q.z, pp.x, pp.y, pp.z);
            if (d <= r2) {
                double4 pd = sdir[idx];
                double wt = filter_wt(pfilter, d, r2);
                double pwt = wt * pw;
                double cos0 = dot(n, mk3(pd.x, pd.y, pd.z));
                double pw2 = cos0 < 0.0 ? pwt * -cos0 : 0.0;
                int wl = (int)(((unsigned long long)__double_as_longlong(pp.w)) >> 40);
                if (wl == 0) s0 += pw2; else if (wl == 1) s1 += pw2; else s2 += pw2;
            }
        });
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (lane_id() == 0) {
            double k = ONE_PI_D / r2;
            if (mode == 0) {
                double *px = out.pass_img + 3 * (long long)h.pixel;
                atomicAdd(px, h.w[0] * (s0 * k));
                atomicAdd(px + 1, h.w[1] * (s1 * k));
                atomicAdd(px + 2, h.w[2] * (s2 * k));
            } else {
                out.out_rgb[3 * qi] = s0 * k;
                out.out_rgb[3 * qi + 1] = s1 * k;
                out.out_rgb[3 * qi + 2] = s2 * k;
            }
        }
    }
}

#endif  // PPM_BUILD_F64

// ---------------------------------------------------------------------------
// FP32 gather over the sorted float4 map with Kahan-compensated per-lane
// flux sums.  Membership: FP32 distance test; candidates inside the rounding
// band [r2_lo, r2_hi] are re-decided by the FP64 predicate on the same
// (f32-valued) coordinates, so the in-radius set equals the f64 one.
// ---------------------------------------------------------------------------
struct Kahan {
    float s, c;
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// pairwise (tree) sum of the lanes' partial sums
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// float -> double that the compiler cannot hoist out of a branch (an inline
// cvt marked volatile): the gathers' FP64 rechecks of the query position sit
// in branches almost never taken, and hoisted to once per query the
// conversions cost FP64 issue slots on every query.
__device__ __forceinline__ double f2d_here(float x) {
    double d;
    asm volatile("cvt.f64.f32 %0, %1;" : "=d"(d) : "f"(x));
    return d;
}

// the kdtree crate's f64 predicate for a candidate in the FP32 rounding band
__device__ __forceinline__ void in_recheck(bool &in, double qx, double qy, double qz, double px, double py, double pz,
                                           double r2) {
    in = sq_euclid(qx, qy, qz, px, py, pz) <= r2;
}

__device__ __forceinline__ bool in_radius_f32(float qx, float qy, float qz, float4 pp, float r2_lo, float r2_hi,
                                              double r2, float &d2f) {
    float dx = qx - pp.x, dy = qy - pp.y, dz = qz - pp.z;
    d2f = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    if (d2f < r2_lo) return true;
    if (d2f > r2_hi) return false;
    return sq_euclid(f2d_here(qx), f2d_here(qy), f2d_here(qz), (double)pp.x, (double)pp.y, (double)pp.z) <= r2;
}

__device__ __forceinline__ float filter_wt_f(int pfilter, float d, float r2) {
    if (pfilter == PF_CONE) {
        float d2 = sqrtf(d / r2) * (1.0f / 1.1f);
        return d2 > 1.0f ? 0.0f : (1.0f - d2) * (float)(1.0 / (1.0 - 2.0 / (3.0 * 1.1)));
    }
    if (pfilter == PF_GAUSS) {
        float e_r = 1.0f - __expf(-1.953f * d / (r2 * 2.0f));
        const float eb = (float)(1.0 - 0.14184788965323);
        return e_r > eb ? 0.0f : 0.918f * (1.0f - e_r / eb) + 0.5f;
    }
    return 1.0f;
}

// a hit point (40 B; its arrays start 256-byte aligned, so every element is
// 8-byte aligned) as five 8-byte loads
static_assert(sizeof(HitPoint<float>) == 40, "five float2 per hit point");
__device__ __forceinline__ HitPoint<float> load_hit(const HitPoint<float> *p) {
    const float2 *v = reinterpret_cast<const float2 *>(p);
    const float2 a = v[0], b = v[1], c = v[2], d = v[3], e = v[4];
    HitPoint<float> h;
    h.pos[0] = a.x; h.pos[1] = a.y; h.pos[2] = b.x;
    h.nrm[0] = b.y; h.nrm[1] = c.x; h.nrm[2] = c.y;
    h.w[0] = d.x; h.w[1] = d.y; h.w[2] = e.x;
    h.pixel = __float_as_int(e.y);
    return h;
}

// Parity export of the render gather, one record per hit point: the FP32
// flux sums per wavelength before the hit point's weight and the pass's
// pw / (pi r^2) scale them, the number of photons found in radius, and the
// sum over those photons of slot_mix(map slot), a checksum of the set.
struct GatherDump {
    float s[3];
    uint32_t count;
    unsigned long long hash;
};
static_assert(sizeof(GatherDump) == 24, "export record layout");

// SplitMix64's output function (Steele, Lea and Flood, OOPSLA 2014) over
// (slot + 1) times its increment: a well-mixed 64-bit value per map slot, so
// that a sum over a set changes when any member does
__host__ __device__ __forceinline__ unsigned long long slot_mix(uint32_t slot) {
    unsigned long long z = ((unsigned long long)slot + 1ull) * 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct GatherOutF {
    float *gathered;     // render: per-pass gathered flux W * sum (normalised later in FP64)
    double *out_rgb;     // estimate entry: per-query radiance
    unsigned long long *count;
    GatherDump *dump;    // render parity export (null in the production render)
};

// a queued part of a tile gather walk (see k_gather_tile)
struct TileItem {
    uint32_t qi0, mask;   // the chunk's first hit point and the group's lanes
    float lo[3], hi[3];   // the group's box
    int32_t row0;         // the slab's first row
    uint32_t b0, b1;      // its batches [b0, b1)
    uint32_t pad;
};
static_assert(sizeof(TileItem) == 48, "queue item layout");

struct TileQueue {
    TileItem *items;
    unsigned long long cap;
};


#if defined(PPM_BUILD_F32)
// Two hit points of the render gather in one warp.  Consecutive hit points
// are mostly neighbouring pixels, a few thousandths apart against radii of
// a few hundredths, so they usually share a cell: then the warp walks the
// union of their rows once and tests every photon against both, sharing
// the photon's load, its index arithmetic and its direction decode, and
// the per-query row set-up.  Returns false (nothing done) when the two are
// in different cells.  Membership, weights and sums are those of the
// one-query walk.
template <bool COUNT, bool DUMP>
__device__ __forceinline__ bool gather_pair(const GridParams &g, double r2, const HitPoint<float> *hp,
                                            const uint32_t *start, const float4 *smap, int pfilter,
                                            const GatherOutF &out, unsigned long long qi) {
    V3<float> qa, qb, na, nb;
    {
        const HitPoint<float> ha = load_hit(hp), hb = load_hit(hp + 1);
        qa = ld3(ha.pos);
        qb = ld3(hb.pos);
        na = ld3(ha.nrm);
        nb = ld3(hb.nrm);
    }
    int c[3], lo[3], hi[3];
    query_cells(g, qa, g.ext, g.extx, c, lo, hi);
    // One set of rows over both queries' cell ranges: y and z cells at most
    // one apart (one more row or column of rows), x cells at most a
    // radius apart.  Each query still culls every row to its own chord.
    const int cb[3] = {CellMath<float>::coord(g, qb.x, 0), CellMath<float>::coord(g, qb.y, 1),
                       CellMath<float>::coord(g, qb.z, 2)};
    if (abs(cb[0] - c[0]) > g.extx || abs(cb[1] - c[1]) > 1 || abs(cb[2] - c[2]) > 1) return false;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int e = a == 0 ? g.extx : g.ext;
        lo[a] = max(min(c[a], cb[a]) - e, 0);
        hi[a] = min(max(c[a], cb[a]) + e, g.dim[a] - 1);
    }
    const float r2f = g.r2f, r2_lo = g.r2_lo, r2_hi = g.r2_hi;
    const unsigned lane = lane_id();
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, b0 = 0.f, b1 = 0.f, b2 = 0.f;
    unsigned long long c_slots = 0, c_valid = 0, c_hits = 0;
    uint32_t na_in = 0, nb_in = 0;             // export only
    unsigned long long ha_in = 0, hb_in = 0;   // export only
    const int ny = hi[1] - lo[1] + 1, nrows = ny * (hi[2] - lo[2] + 1);
    const unsigned le = lanemask_le();
    for (int row0 = 0; row0 < nrows; row0 += 32) {
        // lane's row: the union of the two queries' chord ranges
        uint32_t rbeg = 0, rlen = 0;
        const int row = row0 + (int)lane;
        if (row < nrows) {
            const int zi = __float2int_rz(__fdividef((float)row + 0.5f, (float)ny));   // as make_rows
            const int yy = lo[1] + (row - zi * ny), zz = lo[2] + zi;
            int xa0, xa1, xb0, xb1;
            const bool ra = RowCull<float>::range(g, qa, r2f, yy, zz, lo[0], hi[0], xa0, xa1);
            const bool rb = RowCull<float>::range(g, qb, r2f, yy, zz, lo[0], hi[0], xb0, xb1);
            if (ra || rb) {
                const int x0 = ra ? (rb ? min(xa0, xb0) : xa0) : xb0;
                const int x1 = ra ? (rb ? max(xa1, xb1) : xa1) : xb1;
                const int base = (zz * g.dim[1] + yy) * g.dim[0];
                rbeg = start[base + x0];
                rlen = start[base + x1 + 1] - rbeg;
            }
        }
        const unsigned nonempty = __ballot_sync(0xffffffffu, rlen > 0);
        if (nonempty == 0u) continue;
        const PackedRows pr = pack_rows(rbeg, rlen, nonempty);
        int kbase = -1;
        {
            for (uint32_t win = 0; win < pr.total; win += 32) {
                bool v;
                const uint32_t slot = packed_slot(pr, win, le, kbase, v);
                const float4 p = __ldg(&smap[slot]);
                float dx = qa.x - p.x, dy = qa.y - p.y, dz = qa.z - p.z;
                const float da = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                dx = qb.x - p.x;
                dy = qb.y - p.y;
                dz = qb.z - p.z;
                const float db = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                bool ia = v && da < r2_lo, ib = v && db < r2_lo;
                const bool ba = v && !ia && da <= r2_hi, bb = v && !ib && db <= r2_hi;
                if (__any_sync(0xffffffffu, ba || bb)) {   // FP64 recheck within rounding of r
                    const double px = p.x, py = p.y, pz = p.z;
                    if (ba) in_recheck(ia, f2d_here(qa.x), f2d_here(qa.y), f2d_here(qa.z), px, py, pz, r2);
                    if (bb) in_recheck(ib, f2d_here(qb.x), f2d_here(qb.y), f2d_here(qb.z), px, py, pz, r2);
                }
                if (COUNT) {
                    c_slots += 1;
                    c_valid += 2 * (int)v;
                    c_hits += (int)ia + (int)ib;
                }
                if (DUMP && (ia || ib)) {
                    const unsigned long long hm = slot_mix(slot);
                    na_in += ia ? 1u : 0u;
                    nb_in += ib ? 1u : 0u;
                    ha_in += ia ? hm : 0ull;
                    hb_in += ib ? hm : 0ull;
                }
                if (ia || ib) {
                    const uint32_t mm = __float_as_uint(p.w);
                    float inv;
                    const V3<float> d = oct_raw(mm, inv);
                    const float ca = (na.x * d.x + na.y * d.y + na.z * d.z) * inv;
                    const float cb = (nb.x * d.x + nb.y * d.y + nb.z * d.z) * inv;
                    float wa = (ia && ca < 0.0f) ? -ca : 0.0f, wb = (ib && cb < 0.0f) ? -cb : 0.0f;
                    if (pfilter != PF_NONE) {
                        wa *= filter_wt_f(pfilter, da, r2f);
                        wb *= filter_wt_f(pfilter, db, r2f);
                    }
                    const uint32_t l = mm >> 30;
                    a0 += l == 0u ? wa : 0.0f;
                    a1 += l == 1u ? wa : 0.0f;
                    a2 += l >= 2u ? wa : 0.0f;
                    b0 += l == 0u ? wb : 0.0f;
                    b1 += l == 1u ? wb : 0.0f;
                    b2 += l >= 2u ? wb : 0.0f;
                }
            }
        }
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            c_slots += __shfl_xor_sync(0xffffffffu, c_slots, o);
            c_valid += __shfl_xor_sync(0xffffffffu, c_valid, o);
            c_hits += __shfl_xor_sync(0xffffffffu, c_hits, o);
        }
        if (lane == 0) {
            atomicAdd(out.count + 0, c_valid);
            atomicAdd(out.count + 1, c_hits);
            atomicAdd(out.count + 2, c_slots);
        }
    }
    if (!DUMP) {
        // Six sums over the warp in 15 shuffles: one exchange leaves hit a's
        // three partial sums (lanes l and l + 16) on lanes 0-15 and hit b's
        // on lanes 16-31, then each half sums its three; lanes 0 and 16
        // scale by their hit point's weights and add to its pixel.
        const bool upper = lane >= 16u;
        float s0 = upper ? b0 : a0, s1 = upper ? b1 : a1, s2 = upper ? b2 : a2;
        s0 += __shfl_xor_sync(0xffffffffu, upper ? a0 : b0, 16);
        s1 += __shfl_xor_sync(0xffffffffu, upper ? a1 : b1, 16);
        s2 += __shfl_xor_sync(0xffffffffu, upper ? a2 : b2, 16);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if ((lane & 15u) == 0u) {
            // weights and pixel re-read here (cached) rather than held through the walk
            const HitPoint<float> h = load_hit(hp + (lane >> 4));
            float *px = out.gathered + 3 * (size_t)h.pixel;
            atomicAdd(px, h.w[0] * s0);
            atomicAdd(px + 1, h.w[1] * s1);
            atomicAdd(px + 2, h.w[2] * s2);
        }
        return true;
    }
    // the parity export: every sum reduced on every lane, written with the
    // pair's in-radius counts and checksums
    a0 = warp_sum(a0); a1 = warp_sum(a1); a2 = warp_sum(a2);
    b0 = warp_sum(b0); b1 = warp_sum(b1); b2 = warp_sum(b2);
    {
        for (int o = 16; o > 0; o >>= 1) {
            na_in += __shfl_xor_sync(0xffffffffu, na_in, o);
            nb_in += __shfl_xor_sync(0xffffffffu, nb_in, o);
            ha_in += __shfl_xor_sync(0xffffffffu, ha_in, o);
            hb_in += __shfl_xor_sync(0xffffffffu, hb_in, o);
        }
        if (lane == 0) {
            out.dump[qi] = GatherDump{{a0, a1, a2}, na_in, ha_in};
            out.dump[qi + 1] = GatherDump{{b0, b1, b2}, nb_in, hb_in};
        }
    }
    if (lane == 0) {
        // weights and pixels re-read here (cached) rather than held through the walk
        const HitPoint<float> ha = load_hit(hp), hb = load_hit(hp + 1);
        float *pa = out.gathered + 3 * (size_t)ha.pixel, *pb = out.gathered + 3 * (size_t)hb.pixel;
        atomicAdd(pa, ha.w[0] * a0);
        atomicAdd(pa + 1, ha.w[1] * a1);
        atomicAdd(pa + 2, ha.w[2] * a2);
        atomicAdd(pb, hb.w[0] * b0);
        atomicAdd(pb + 1, hb.w[1] * b1);
        atomicAdd(pb + 2, hb.w[2] * b2);
    }
    return true;
}
#endif

#if defined(PPM_BUILD_F32)
// The render gather, row-walk form (the default): one warp per hit point,
// or per two hit points of one cell (gather_pair).  Warps take their hit
// points from a counter, two at a time, so the hit points in flight are a
// narrow window of the list (appended in pixel tiles by the eye pass): neighbouring warps read the
// same photons, from L1 or L2, and a slow warp does not hold up the rest
// (measured on the glass box: 0.402 ms against 0.406 for 1, 0.410 for 4 and
// 0.43 for 8 or a fixed warp stride).  Five blocks per SM (at most 51
// registers; it needs 46 without spilling) measured 1 % faster than four.
// One step of the row walk: hit points qi and qi + 1 in one walk when both
// are left and share a cell (returns 2), else hit point qi alone (returns
// 1).  All lanes of the warp enter with the same arguments.
template <bool COUNT, bool DUMP>
__device__ __forceinline__ unsigned gather_step(const GridParams &g, double r2, const HitPoint<float> *hits,
                                                unsigned long long qi, unsigned long long left,
                                                const uint32_t *start, const float4 *smap, int pfilter,
                                                const GatherOutF &out) {
    if (left == 2 && gather_pair<COUNT, DUMP>(g, r2, hits + qi, start, smap, pfilter, out, qi)) return 2u;
    const unsigned lane = lane_id();
    const HitPoint<float> h = load_hit(hits + qi);
    const float r2_lo = g.r2_lo, r2_hi = g.r2_hi, r2f = g.r2f;
    V3<float> q = ld3(h.pos), n = ld3(h.nrm);
    int c[3], lo[3], hi[3];
    query_cells(g, q, g.ext, g.extx, c, lo, hi);
    // Per-lane sums: a lane adds a few dozen terms (relative error <
    // 1e-6), and the three sums take the photon's value or zero without
    // a branch on its wavelength.
    float k0 = 0.f, k1 = 0.f, k2 = 0.f;
    unsigned long long c_slots = 0, c_valid = 0, c_hits = 0;
    uint32_t d_in = 0;             // export only
    unsigned long long d_hash = 0;   // export only
    {
        for_each_candidate_two(g, start, q, r2f, lo, hi, smap,
                               [&](auto two, float4 p0, bool v0, uint32_t i0, float4 p1, bool v1, uint32_t i1) {
            constexpr bool TWO = decltype(two)::value;
            if (COUNT) {
                c_slots += TWO ? 2 : 1;
                c_valid += (int)v0 + (int)v1;
            }
            float dx = q.x - p0.x, dy = q.y - p0.y, dz = q.z - p0.z;
            const float d0 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
            float d1 = 0.0f;
            if constexpr (TWO) {
                dx = q.x - p1.x;
                dy = q.y - p1.y;
                dz = q.z - p1.z;
                d1 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
            }
            // in_radius_f32 on both: below r2_lo in, above r2_hi out, between in FP64.
            // The vote keeps the FP64 recheck a branch that warps almost never
            // take; left to the compiler it was predicated into every step,
            // which costs issue slots on this GPU's narrow FP64 pipe.
            bool in0 = v0 && d0 < r2_lo, in1 = TWO && v1 && d1 < r2_lo;
            const bool b0 = v0 && !in0 && d0 <= r2_hi, b1 = TWO && v1 && !in1 && d1 <= r2_hi;
            if (__any_sync(0xffffffffu, b0 || b1)) {
                const double qx = f2d_here(q.x), qy = f2d_here(q.y), qz = f2d_here(q.z);
                if (b0) in0 = sq_euclid(qx, qy, qz, (double)p0.x, (double)p0.y, (double)p0.z) <= r2;
                if (b1) in1 = sq_euclid(qx, qy, qz, (double)p1.x, (double)p1.y, (double)p1.z) <= r2;
            }
            if (in0 || in1) {
                const uint32_t m0 = __float_as_uint(p0.w), m1 = __float_as_uint(p1.w);
                const float c0 = oct_dot(m0, n);
                const float c1 = TWO ? oct_dot(m1, n) : 0.0f;
                float w0 = (in0 && c0 < 0.0f) ? -c0 : 0.0f, w1 = (in1 && c1 < 0.0f) ? -c1 : 0.0f;
                if (pfilter != PF_NONE) {
                    w0 *= filter_wt_f(pfilter, d0, r2f);
                    if (TWO) w1 *= filter_wt_f(pfilter, d1, r2f);
                }
                const uint32_t l0 = m0 >> 30, l1 = m1 >> 30;
                if constexpr (TWO) {
                    k0 += (l0 == 0u ? w0 : 0.0f) + (l1 == 0u ? w1 : 0.0f);
                    k1 += (l0 == 1u ? w0 : 0.0f) + (l1 == 1u ? w1 : 0.0f);
                    k2 += (l0 >= 2u ? w0 : 0.0f) + (l1 >= 2u ? w1 : 0.0f);
                } else {
                    k0 += l0 == 0u ? w0 : 0.0f;
                    k1 += l0 == 1u ? w0 : 0.0f;
                    k2 += l0 >= 2u ? w0 : 0.0f;
                }
                if (COUNT) c_hits += (int)in0 + (int)in1;
                if (DUMP) {
                    d_in += (in0 ? 1u : 0u) + (in1 ? 1u : 0u);
                    d_hash += (in0 ? slot_mix(i0) : 0ull) + (in1 ? slot_mix(i1) : 0ull);
                }
            }
        });
    }
    const float s0 = warp_sum(k0), s1 = warp_sum(k1), s2 = warp_sum(k2);
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            c_slots += __shfl_xor_sync(0xffffffffu, c_slots, o);
            c_valid += __shfl_xor_sync(0xffffffffu, c_valid, o);
            c_hits += __shfl_xor_sync(0xffffffffu, c_hits, o);
        }
        if (lane == 0) {
            atomicAdd(out.count + 0, c_valid);
            atomicAdd(out.count + 1, c_hits);
            atomicAdd(out.count + 2, c_slots);
        }
    }
    if constexpr (DUMP) {
        for (int o = 16; o > 0; o >>= 1) {
            d_in += __shfl_xor_sync(0xffffffffu, d_in, o);
            d_hash += __shfl_xor_sync(0xffffffffu, d_hash, o);
        }
        if (lane == 0) out.dump[qi] = GatherDump{{s0, s1, s2}, d_in, d_hash};
    }
    if (lane == 0) {
        // FP32 only here: an FP64 instruction costs a warp-wide slot of
        // the narrow FP64 pipe even with one active lane
        float *px = out.gathered + 3 * (size_t)h.pixel;
        atomicAdd(px, h.w[0] * s0);
        atomicAdd(px + 1, h.w[1] * s1);
        atomicAdd(px + 2, h.w[2] * s2);
    }
    return 1u;
}

template <bool COUNT, bool DUMP = false>
__global__ void __launch_bounds__(256, 5) k_gather_f(const HitPoint<float> *hits, PassState *st, long long n_fixed,
                                                     const float4 *smap, const uint32_t *start, int pfilter,
                                                     GatherOutF out) {
    constexpr unsigned CHUNK = 2u;
    grid_dependency_wait();   // a programmatic dependent of the map's scatter
    const unsigned long long nq = n_hitpoints(st, n_fixed);
    const GridParams g = st->grid;
    const unsigned lane = lane_id();
    unsigned long long qi = 0ull, qend = 0ull;
    for (;;) {
        if (qi == qend) {
            unsigned long long c = 0;
            if (lane == 0) c = atomicAdd(&st->gather_next, (unsigned long long)CHUNK);
            c = __shfl_sync(0xffffffffu, c, 0);
            if (c >= nq) break;
            qi = c;
            qend = c + CHUNK < nq ? c + CHUNK : nq;
        }
        qi += gather_step<COUNT, DUMP>(g, st->r2, hits, qi, qend - qi, start, smap, pfilter, out);
    }
    grid_dependents_launch();
}

// ---------------------------------------------------------------------------
// Render gather, tile form.  A warp takes 32 consecutive hit points, one per
// lane; the eye pass appends them in pixel tiles, so they are a compact
// patch of the scene.  The warp walks the photons of the cell rows around
// all of them once: each batch of 32 photons is loaded (one coalesced
// 512-byte read), decoded once (position, unit direction, wavelength) and
// staged in shared memory grouped by wavelength, and then every lane tests
// every staged photon against its own hit point.  A test is a distance, a
// compare and, in radius, a cosine added to the lane's sum of that
// wavelength: no per-hit-point row set-up, no idle lanes at row ends, no
// warp reduction.  Rows are laid end to end, so batches are full until the
// last.  Membership is exactly the kdtree crate's f64 predicate: FP32 d^2
// below the FP32 band [r2_lo, r2_hi] is in, above it out, and a batch in
// which any lane met a photon inside the band is redone with those photons
// re-decided in FP64 (one warp vote per batch; the band is 2e-6 r^2 wide).
// Flux: per-batch FP32 partial sums (at most 32 terms) added to per-lane
// Kahan-compensated totals.
//
// A chunk whose hit points are spread out (an object edge inside the tile,
// reflected or refracted hit points) is split into groups of hit points
// within 2r of a leader per axis, each walked on its own; the lanes outside
// the current group carry a far-away position, so they find nothing.
// ---------------------------------------------------------------------------
#if defined(PPM_BUILD_F32)
constexpr int GATHER_TILE_WARPS = 8;   // warps per block

// Rows (y, z) and their culled x ranges around the box [lo, hi]: the box's
// distance to the row's y/z slab bounds the chord of every member's sphere
// in that row, so the row keeps the cells within that chord of the box (with
// the margins of RowCull, which exceed the rounding of cell coordinates).
__device__ __forceinline__ bool box_row_range(const GridParams &g, V3<float> lo, V3<float> hi, float r2, int yy,
                                              int zz, int lo_x, int hi_x, int &x0, int &x1) {
    const float c = g.cellf, m = 4e-3f * c;
    const float ylo = g.orgf[1] + (float)yy * c, zlo = g.orgf[2] + (float)zz * c;
    const float dy = fmaxf(0.0f, fmaxf(ylo - hi.y, lo.y - (ylo + c)) - m);
    const float dz = fmaxf(0.0f, fmaxf(zlo - hi.z, lo.z - (zlo + c)) - m);
    const float rem = r2 * 1.00002f - dy * dy - dz * dz;
    if (rem < 0.0f) return false;
    const float rx = sqrtf(rem) * 1.00001f;
    const float fx0 = floorf((lo.x - rx - g.orgf[0]) * g.invxf - 4e-3f);
    const float fx1 = floorf((hi.x + rx - g.orgf[0]) * g.invxf + 4e-3f);
    x0 = max(lo_x, (int)fmaxf(fx0, -1.0f));
    x1 = min(hi_x, (int)fminf(fx1, (float)g.dim[0]));
    return x0 <= x1;
}

template <int FILTER>
__device__ __forceinline__ float tile_filter(float d2, float r2f) {
    if constexpr (FILTER == PF_NONE) return 1.0f;
    else return filter_wt_f(FILTER, d2, r2f);
}

// the group's box and its cells, shared by the warp's lanes through shared
// memory (they are needed once per 32 rows, not in the test loop)
struct TileBox {
    float lo[3], hi[3];
    float r2;   // the group's largest radius^2 (estimate entry point)
    int cx0, cx1, cy0, cz0, ny, nrows;
};

// A group's walk is capped: the warp walks at most TILE_SPLIT batches of each
// row slab of its group itself and queues the rest of the slab as items of
// TILE_SPLIT batches, which k_gather_tile_items takes up after all chunks
// are done.  A few dense chunks (caustics) hold far more photons than the
// rest; uncapped, they decide when the launch ends.  Every walk adds its
// part of a hit point's sums to the pixel with FP32 atomics (the estimate is
// linear in the photons), so a split walk gives the same sums up to the
// order of the additions.  A full queue is never an error: the warp then
// walks the item itself.
constexpr uint32_t TILE_SPLIT = 8;

// per-lane counters of the counting and export variants
struct TileCount {
    uint32_t d_in = 0;
    unsigned long long d_hash = 0, tests = 0, slots = 0, hits = 0;
};

// the box's cell ranges (one lane; box.lo / hi set)
__device__ __forceinline__ void tile_box_cells(const GridParams &g, TileBox &box) {
    box.cx0 = max(CellMath<float>::coord(g, box.lo[0], 0) - g.extx, 0);
    box.cx1 = min(CellMath<float>::coord(g, box.hi[0], 0) + g.extx, g.dim[0] - 1);
    box.cy0 = max(CellMath<float>::coord(g, box.lo[1], 1) - g.ext, 0);
    const int cy1 = min(CellMath<float>::coord(g, box.hi[1], 1) + g.ext, g.dim[1] - 1);
    box.cz0 = max(CellMath<float>::coord(g, box.lo[2], 2) - g.ext, 0);
    const int cz1 = min(CellMath<float>::coord(g, box.hi[2], 2) + g.ext, g.dim[2] - 1);
    box.ny = cy1 - box.cy0 + 1;
    box.nrows = box.ny * (cz1 - box.cz0 + 1);
}

// Batches [b_begin, b_end) of the row slab that starts at row0 (32 rows of
// the box, end to end); returns the slab's batch count.  Lanes outside the
// group carry a far-away q.
template <bool COUNT, bool DUMP, int FILTER>
__device__ __forceinline__ uint32_t tile_walk(const GridParams &g, const TileBox &box, int row0, uint32_t b_begin,
                                              uint32_t b_end, const uint32_t *start, const float4 *smap, float4 *sp,
                                              float4 *sd, V3<float> q, V3<float> n, bool member, double r2, Kahan &k0,
                                              Kahan &k1, Kahan &k2, TileCount &cn) {
    const unsigned lane = lane_id(), lt = (1u << lane) - 1u;
    const float r2f = g.r2f, r2_lo = g.r2_lo, r2_hi = g.r2_hi;
    const int nrows = box.nrows;
    uint32_t rbeg = 0, rlen = 0;
    const int row = row0 + (int)lane;
    if (row < nrows) {
        const int ny = box.ny;
        const int zz = box.cz0 + row / ny, yy = box.cy0 + row % ny;
        int x0, x1;
        if (box_row_range(g, mk3(box.lo[0], box.lo[1], box.lo[2]), mk3(box.hi[0], box.hi[1], box.hi[2]), r2f, yy, zz,
                          box.cx0, box.cx1, x0, x1)) {
            const int base = (zz * g.dim[1] + yy) * g.dim[0];
            rbeg = start[base + x0];
            rlen = start[base + x1 + 1] - rbeg;
        }
    }
    uint32_t incl = rlen;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += u;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t excl = incl - rlen;
    const uint32_t nb = (total + 31) / 32;
    const uint32_t bend = b_end < nb ? b_end : nb;
    for (uint32_t bi = b_begin; bi < bend; bi++) {
        // this lane's photon: the row r with excl_r <= j < incl_r
        const uint32_t j = bi * 32 + lane;
        int r = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
            if (__shfl_sync(0xffffffffu, incl, r + step - 1) <= j) r += step;
        const uint32_t rb = __shfl_sync(0xffffffffu, rbeg, r), rx = __shfl_sync(0xffffffffu, excl, r);
        const bool v = j < total;
        uint32_t wl = 3u;
        float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pd = pa;
        if (v) {
            const uint32_t slot = rb + (j - rx);
            const float4 p = __ldg(&smap[slot]);
            const uint32_t m = __float_as_uint(p.w);
            float inv;
            const V3<float> d = oct_raw(m, inv);
            pa = make_float4(p.x, p.y, p.z, __uint_as_float(slot));
            pd = make_float4(-d.x * inv, -d.y * inv, -d.z * inv, 0.f);
            wl = min(m >> 30, 2u);
        }
        // stage grouped by wavelength
        const unsigned m0 = __ballot_sync(0xffffffffu, wl == 0u), m1 = __ballot_sync(0xffffffffu, wl == 1u),
                       m2 = __ballot_sync(0xffffffffu, wl == 2u);
        const int n0 = __popc(m0), n01 = n0 + __popc(m1), nv = n01 + __popc(m2);
        if (v) {
            const int at = wl == 0u ? __popc(m0 & lt) : (wl == 1u ? n0 + __popc(m1 & lt) : n01 + __popc(m2 & lt));
            sp[at] = pa;
            sd[at] = pd;
        }
        __syncwarp();
        // the tests; EXACT re-decides band photons in FP64
        bool band = false;
        auto sweep = [&](auto exact, int t0, int t1) -> float {
            constexpr bool EXACT = decltype(exact)::value;
            float acc = 0.0f;
#pragma unroll 2
            for (int t = t0; t < t1; t++) {
                const float4 a = sp[t], b = sd[t];
                const float dx = q.x - a.x, dy = q.y - a.y, dz = q.z - a.z;
                const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                bool in = d2 < r2_lo;
                const bool bd = !in && d2 <= r2_hi;
                if constexpr (EXACT) {
                    if (bd) in = sq_euclid(f2d_here(q.x), f2d_here(q.y), f2d_here(q.z), (double)a.x, (double)a.y,
                                           (double)a.z) <= r2;
                } else {
                    band |= bd;
                }
                const float c = __fmaf_rn(n.z, b.z, __fmaf_rn(n.y, b.y, n.x * b.x));
                float w = in ? fmaxf(c, 0.0f) : 0.0f;
                if constexpr (FILTER != PF_NONE) w *= in ? tile_filter<FILTER>(d2, r2f) : 0.0f;
                acc += w;
                if constexpr (EXACT && (DUMP || COUNT)) {
                    if (in) {
                        if (DUMP) { cn.d_in += 1u; cn.d_hash += slot_mix(__float_as_uint(a.w)); }
                        if (COUNT) cn.hits += 1;
                    }
                }
            }
            return acc;
        };
        float a0 = sweep(std::false_type{}, 0, n0);
        float a1 = sweep(std::false_type{}, n0, n01);
        float a2 = sweep(std::false_type{}, n01, nv);
        if (__any_sync(0xffffffffu, band) || DUMP || COUNT) {
            // exact pass: the same tests with band photons re-decided in FP64
            // (the export and the counters always take it, as they count members)
            a0 = sweep(std::true_type{}, 0, n0);
            a1 = sweep(std::true_type{}, n0, n01);
            a2 = sweep(std::true_type{}, n01, nv);
        }
        k0.add(a0);
        k1.add(a1);
        k2.add(a2);
        if (COUNT) {
            cn.tests += member ? (unsigned long long)nv : 0ull;   // photon-hit point distance tests
            cn.slots += (unsigned long long)nv;                   // lane slots the batch issued
        }
        __syncwarp();   // the next batch overwrites the stage
    }
    return nb;
}

// a member lane's sums into its pixel (and into its export record)
template <bool DUMP>
__device__ __forceinline__ void tile_flush(const HitPoint<float> *hits, unsigned long long qi, const Kahan &k0,
                                           const Kahan &k1, const Kahan &k2, const TileCount &cn,
                                           const GatherOutF &out) {
    const float s0 = k0.s - k0.c, s1 = k1.s - k1.c, s2 = k2.s - k2.c;
    const HitPoint<float> h = load_hit(hits + qi);
    float *px = out.gathered + 3 * (size_t)h.pixel;
    atomicAdd(px, h.w[0] * s0);
    atomicAdd(px + 1, h.w[1] * s1);
    atomicAdd(px + 2, h.w[2] * s2);
    if (DUMP) {
        GatherDump &d = out.dump[qi];
        atomicAdd(&d.s[0], s0);
        atomicAdd(&d.s[1], s1);
        atomicAdd(&d.s[2], s2);
        atomicAdd(&d.count, cn.d_in);
        atomicAdd(&d.hash, cn.d_hash);
    }
}

template <bool COUNT>
__device__ __forceinline__ void tile_count_flush(TileCount &cn, const GatherOutF &out) {
    if (!COUNT) return;
    for (int o = 16; o > 0; o >>= 1) {
        cn.tests += __shfl_xor_sync(0xffffffffu, cn.tests, o);
        cn.hits += __shfl_xor_sync(0xffffffffu, cn.hits, o);
        cn.slots += __shfl_xor_sync(0xffffffffu, cn.slots, o);
    }
    if (lane_id() == 0) {
        atomicAdd(out.count + 0, cn.tests);
        atomicAdd(out.count + 1, cn.hits);
        atomicAdd(out.count + 2, cn.slots);
    }
}

template <bool COUNT, bool DUMP, int FILTER>
__global__ void __launch_bounds__(32 * GATHER_TILE_WARPS) k_gather_tile(const HitPoint<float> *hits, PassState *st,
                                                                        const float4 *smap, const uint32_t *start,
                                                                        TileQueue queue, GatherOutF out) {
    __shared__ float4 s_pos[GATHER_TILE_WARPS][32];   // x, y, z, map slot (export only)
    __shared__ float4 s_dir[GATHER_TILE_WARPS][32];   // -direction (unit)
    __shared__ float4 s_own[GATHER_TILE_WARPS][32];   // each lane's hit point position
    __shared__ TileBox s_box[GATHER_TILE_WARPS];
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    float4 *const sp = s_pos[wid], *const sd = s_dir[wid];
    TileBox &box = s_box[wid];
    const unsigned long long nq = n_hitpoints(st, -1);
    const GridParams g = st->grid;
    const double r2 = st->r2;
    const float two_r = 2.0f * sqrtf(g.r2f) * 1.001f;
    constexpr float FAR = 1e30f;   // position of lanes outside the group: no photon is within r of it
    TileCount cn;
    for (;;) {
        unsigned long long c0 = 0;
        if (lane == 0) c0 = atomicAdd(&st->gather_next, 32ull);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        if (c0 >= nq) break;
        const unsigned long long qi = c0 + lane;
        const bool valid = qi < nq;
        V3<float> n = mk3(0.f, 0.f, 0.f);
        {
            float4 own = make_float4(FAR, FAR, FAR, 0.f);
            if (valid) {
                const HitPoint<float> h = load_hit(hits + qi);
                own = make_float4(h.pos[0], h.pos[1], h.pos[2], 0.f);
                n = ld3(h.nrm);
            }
            s_own[wid][lane] = own;
        }
        Kahan k0 = {0.f, 0.f}, k1 = {0.f, 0.f}, k2 = {0.f, 0.f};
        unsigned pending = __ballot_sync(0xffffffffu, valid);
        while (pending) {
            // the group: pending lanes within 2r of the leader on every axis
            const int leader = __ffs(pending) - 1;
            __syncwarp();
            const float4 own = s_own[wid][lane], ld = s_own[wid][leader];
            const bool member = ((pending >> lane) & 1u) && fabsf(own.x - ld.x) <= two_r &&
                                fabsf(own.y - ld.y) <= two_r && fabsf(own.z - ld.z) <= two_r;
            const unsigned gmask = __ballot_sync(0xffffffffu, member);
            pending &= ~gmask;
            const V3<float> q = member ? mk3(own.x, own.y, own.z) : mk3(FAR, FAR, FAR);
            {
                V3<float> lo = q, hi = member ? q : mk3(-FAR, -FAR, -FAR);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    lo.x = fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
                    lo.y = fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
                    lo.z = fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
                    hi.x = fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
                    hi.y = fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
                    hi.z = fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
                }
                if (lane == 0) {
                    box.lo[0] = lo.x; box.lo[1] = lo.y; box.lo[2] = lo.z;
                    box.hi[0] = hi.x; box.hi[1] = hi.y; box.hi[2] = hi.z;
                    tile_box_cells(g, box);
                }
                __syncwarp();
            }
            const int nrows = box.nrows;
            for (int row0 = 0; row0 < nrows; row0 += 32) {
                const uint32_t nb = tile_walk<COUNT, DUMP, FILTER>(g, box, row0, 0, TILE_SPLIT, start, smap, sp, sd, q,
                                                                  n, member, r2, k0, k1, k2, cn);
                for (uint32_t b = TILE_SPLIT; b < nb; b += TILE_SPLIT) {
                    const uint32_t be = b + TILE_SPLIT < nb ? b + TILE_SPLIT : nb;
                    unsigned long long slot = 0;
                    if (lane == 0) slot = atomicAdd(&st->tile_items, 1ull);
                    slot = __shfl_sync(0xffffffffu, slot, 0);
                    if (slot < queue.cap) {
                        if (lane == 0) {
                            TileItem it;
                            it.qi0 = (uint32_t)c0;
                            it.mask = gmask;
                            for (int a = 0; a < 3; a++) { it.lo[a] = box.lo[a]; it.hi[a] = box.hi[a]; }
                            it.row0 = row0;
                            it.b0 = b;
                            it.b1 = be;
                            it.pad = 0;
                            queue.items[slot] = it;
                        }
                    } else {   // queue full: walk it here
                        tile_walk<COUNT, DUMP, FILTER>(g, box, row0, b, be, start, smap, sp, sd, q, n, member, r2, k0,
                                                       k1, k2, cn);
                    }
                }
            }
        }
        if (valid) tile_flush<DUMP>(hits, qi, k0, k1, k2, cn, out);
        cn.d_in = 0;
        cn.d_hash = 0;
        __syncwarp();   // s_own is rewritten by the next chunk
    }
    tile_count_flush<COUNT>(cn, out);
}

// The queued parts of the walks: one item per warp at a time.
template <bool COUNT, bool DUMP, int FILTER>
__global__ void __launch_bounds__(32 * GATHER_TILE_WARPS) k_gather_tile_items(const HitPoint<float> *hits,
                                                                              PassState *st, const float4 *smap,
                                                                              const uint32_t *start, TileQueue queue,
                                                                              GatherOutF out) {
    __shared__ float4 s_pos[GATHER_TILE_WARPS][32];
    __shared__ float4 s_dir[GATHER_TILE_WARPS][32];
    __shared__ TileBox s_box[GATHER_TILE_WARPS];
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    float4 *const sp = s_pos[wid], *const sd = s_dir[wid];
    TileBox &box = s_box[wid];
    const GridParams g = st->grid;
    const double r2 = st->r2;
    const unsigned long long n_items = st->tile_items < queue.cap ? st->tile_items : queue.cap;
    constexpr float FAR = 1e30f;
    TileCount cn;
    for (;;) {
        unsigned long long i = 0;
        if (lane == 0) i = atomicAdd(&st->tile_next, 1ull);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= n_items) break;
        const TileItem it = queue.items[i];
        const bool member = (it.mask >> lane) & 1u;
        const unsigned long long qi = (unsigned long long)it.qi0 + lane;
        V3<float> q = mk3(FAR, FAR, FAR), n = mk3(0.f, 0.f, 0.f);
        if (member) {
            const HitPoint<float> h = load_hit(hits + qi);
            q = ld3(h.pos);
            n = ld3(h.nrm);
        }
        __syncwarp();   // the previous item's walk is done with the box
        if (lane == 0) {
            for (int a = 0; a < 3; a++) { box.lo[a] = it.lo[a]; box.hi[a] = it.hi[a]; }
            tile_box_cells(g, box);
        }
        __syncwarp();
        Kahan k0 = {0.f, 0.f}, k1 = {0.f, 0.f}, k2 = {0.f, 0.f};
        tile_walk<COUNT, DUMP, FILTER>(g, box, it.row0, it.b0, it.b1, start, smap, sp, sd, q, n, member, r2, k0, k1,
                                       k2, cn);
        if (member) tile_flush<DUMP>(hits, qi, k0, k1, k2, cn, out);
        cn.d_in = 0;
        cn.d_hash = 0;
    }
    tile_count_flush<COUNT>(cn, out);
}
#endif  // PPM_BUILD_F32

// ---------------------------------------------------------------------------
// Hit points in Morton order, the tile gather's input.  The eye pass appends
// hit points warp by warp in whatever order its warps run, so 32 consecutive
// hit points are rarely one patch of the scene.  On the eye stream (beside
// the photon trace) the hit points are counting-sorted by the Morton code of
// their cell in a 128^3 grid of cubic cells over their bounds: bounds, key
// and rank per hit point, scan of the 2^21 key counts, placement.  32
// consecutive sorted hit points then lie in one or a few neighbouring cells.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_hit_bounds(const HitPoint<float> *hits, PassState *st) {
    const unsigned long long n = n_hitpoints(st, -1);
    float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const float2 a = reinterpret_cast<const float2 *>(hits + i)[0];
        const float z = reinterpret_cast<const float *>(hits + i)[2];
        const float v[3] = {a.x, a.y, z};
#pragma unroll
        for (int k = 0; k < 3; k++)
            if (v[k] > -3e38f && v[k] < 3e38f) {   // finite (false for NaN)
                lo[k] = fminf(lo[k], v[k]);
                hi[k] = fmaxf(hi[k], v[k]);
            }
    }
    // warp, then block reduction; one atomic per block and bound
    __shared__ float slo[3][8], shi[3][8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        if (lane_id() == 0) { slo[k][threadIdx.x >> 5] = lo[k]; shi[k][threadIdx.x >> 5] = hi[k]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        float l = slo[k][0], h = shi[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            l = fminf(l, slo[k][w]);
            h = fmaxf(h, shi[k][w]);
        }
        if (l <= h) {
            atomicMin(&st->hb_lo[k], ordf_enc(__float_as_uint(l)));
            atomicMax(&st->hb_hi[k], ordf_enc(__float_as_uint(h)));
        }
    }
}

__global__ void __launch_bounds__(256) k_hit_key(const HitPoint<float> *hits, PassState *st, uint32_t *count,
                                                 uint2 *keyrank) {
    const unsigned long long n = n_hitpoints(st, -1);
    float org[3], ext = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        org[k] = ordf_dec(st->hb_lo[k]);
        ext = fmaxf(ext, ordf_dec(st->hb_hi[k]) - org[k]);
    }
    const float inv = ext > 0.0f && ext < 3e38f ? (float)(1 << HIT_MORTON_BITS) / ext : 0.0f;
    const int top = (1 << HIT_MORTON_BITS) - 1;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const float2 a = reinterpret_cast<const float2 *>(hits + i)[0];
        const float z = reinterpret_cast<const float *>(hits + i)[2];
        const float v[3] = {a.x, a.y, z};
        uint32_t key = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float f = (v[k] - org[k]) * inv;   // NaN and out-of-range clamp to the grid
            const int c = f >= 0.0f ? (f < (float)top ? (int)f : top) : 0;
            key |= spread3((uint32_t)c) << (2 - k);
        }
        keyrank[i] = make_uint2(key, atomicAdd(&count[key], 1u));
    }
}

__global__ void __launch_bounds__(256) k_hit_place(const HitPoint<float> *hits, const PassState *st,
                                                   const uint2 *keyrank, const uint32_t *start,
                                                   HitPoint<float> *sorted) {
    const unsigned long long n = n_hitpoints(st, -1);
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 kr = keyrank[i];
        sorted[start[kr.x] + kr.y] = hits[i];
    }
}

// ---------------------------------------------------------------------------
// Estimate entry point (per-query radii, ppm_estimate_f32), chunk form.  A
// warp takes 32 consecutive queries of the cell-sorted batch.  A compact
// chunk -- one whose box, widened by its largest radius, is small beside the
// members' own spheres (dense queries, e.g. inside a caustic blob) -- is
// walked as in the render's tile gather: each photon of the union of the
// members' rows is loaded and decoded once and tested by every lane against
// its own query and radius.  Otherwise the warp estimates its queries one
// after another, its lanes striding through each query's own culled rows.
// Both modes add every flux term w = max(0, -n . dir) in [0, 1] as an
// integer of 2^-23 units (one FFMA puts round(w 2^23) in the mantissa of
// 2^23 + w 2^23), so each query's sum is exact whatever the order, the
// chunking or the mode: a query's estimate depends only on the query.
// ---------------------------------------------------------------------------
constexpr float FIX_ONE = 8388608.0f;                 // 2^23
constexpr uint32_t FIX_BIAS = 0x4b000000u;            // bits of 2^23
constexpr double FIX_UNIT = 1.0 / 8388608.0;          // 2^-23
constexpr float EST_TILE_RATIO = 0.5f;                // tile mode: union box <= this x sum of member cubes

// round(w 2^23) + FIX_BIAS as the bits of one float (w in [0, 1])
__device__ __forceinline__ uint32_t fix_bits(float w) { return __float_as_uint(__fmaf_rn(w, FIX_ONE, FIX_ONE)); }

template <bool COUNT>
__global__ void __launch_bounds__(32 * GATHER_TILE_WARPS, 4) k_estimate_tile(const HitPoint<float> *hits, const double *r2s,
                                                                          long long nq, PassState *st,
                                                                          const float4 *smap, const uint32_t *start,
                                                                          double pw, GatherOutF out) {
    __shared__ float4 s_pos[GATHER_TILE_WARPS][32];
    __shared__ float4 s_dir[GATHER_TILE_WARPS][32];
    __shared__ float4 s_own[GATHER_TILE_WARPS][32];   // x, y, z, radius
    __shared__ TileBox s_box[GATHER_TILE_WARPS];
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    float4 *const sp = s_pos[wid], *const sd = s_dir[wid];
    TileBox &box = s_box[wid];
    const unsigned lt = (1u << lane) - 1u;
    const GridParams g = st->grid;
    constexpr float FAR = 1e30f;
    unsigned long long c_tests = 0, c_slots = 0, c_hits = 0;
    for (;;) {
        unsigned long long c0 = 0;
        if (lane == 0) c0 = atomicAdd(&st->gather_next, 32ull);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        if (c0 >= (unsigned long long)nq) break;
        const unsigned long long qi = c0 + lane;
        const bool valid = qi < (unsigned long long)nq;
        V3<float> n = mk3(0.f, 0.f, 0.f);
        double r2 = 0.0;
        float r2_lo = -1.0f, r2_hi = -1.0f, rad = 0.0f;
        float4 mine = make_float4(FAR, FAR, FAR, 0.f);
        if (valid) {
            const HitPoint<float> h = load_hit(hits + qi);
            r2 = r2s[qi];
            r2_lo = __double2float_rd(r2 * (1.0 - 1e-6));
            r2_hi = __double2float_ru(r2 * (1.0 + 1e-6));
            rad = sqrtf(r2_hi) * 1.000001f;   // at least the radius
            mine = make_float4(h.pos[0], h.pos[1], h.pos[2], rad);
            n = ld3(h.nrm);
        }
        s_own[wid][lane] = mine;
        unsigned long long t0 = 0, t1 = 0, t2 = 0;   // flux sums in 2^-23 units
        // the chunk: compact enough to share one walk?
        float lox = mine.x, loy = mine.y, loz = mine.z;
        float hix = valid ? mine.x : -FAR, hiy = valid ? mine.y : -FAR, hiz = valid ? mine.z : -FAR;
        float rmax = rad, vsum = valid ? 8.0f * rad * rad * rad : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lox = fminf(lox, __shfl_xor_sync(0xffffffffu, lox, o));
            loy = fminf(loy, __shfl_xor_sync(0xffffffffu, loy, o));
            loz = fminf(loz, __shfl_xor_sync(0xffffffffu, loz, o));
            hix = fmaxf(hix, __shfl_xor_sync(0xffffffffu, hix, o));
            hiy = fmaxf(hiy, __shfl_xor_sync(0xffffffffu, hiy, o));
            hiz = fmaxf(hiz, __shfl_xor_sync(0xffffffffu, hiz, o));
            rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
            vsum += __shfl_xor_sync(0xffffffffu, vsum, o);
        }
        const float vunion = (hix - lox + 2.0f * rmax) * (hiy - loy + 2.0f * rmax) * (hiz - loz + 2.0f * rmax);
        unsigned pending = __ballot_sync(0xffffffffu, valid);
        __syncwarp();
        if (vunion <= EST_TILE_RATIO * vsum) {
            while (pending) {
                // the group: pending lanes within 2 rmax of the leader on every axis
                const int leader = __ffs(pending) - 1;
                const float4 own = mine, ld = s_own[wid][leader];
                const float reach = 2.0f * rmax;
                const bool member = ((pending >> lane) & 1u) && fabsf(own.x - ld.x) <= reach &&
                                    fabsf(own.y - ld.y) <= reach && fabsf(own.z - ld.z) <= reach;
                pending &= ~__ballot_sync(0xffffffffu, member);
                const V3<float> q = member ? mk3(own.x, own.y, own.z) : mk3(FAR, FAR, FAR);
                {
                    V3<float> lo = q, hi = member ? q : mk3(-FAR, -FAR, -FAR);
                    float gr = member ? own.w : 0.0f;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        lo.x = fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
                        lo.y = fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
                        lo.z = fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
                        hi.x = fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
                        hi.y = fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
                        hi.z = fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
                        gr = fmaxf(gr, __shfl_xor_sync(0xffffffffu, gr, o));
                    }
                    if (lane == 0) {
                        // cells a radius gr can span (as the per-query walk's ext)
                        const int ext = min(g.ext, max(1, (int)ceilf(gr * g.invf + 3e-3f)));
                        const int extx = min(g.extx, max(1, (int)ceilf(gr * g.invxf + 3e-3f)));
                        box.lo[0] = lo.x; box.lo[1] = lo.y; box.lo[2] = lo.z;
                        box.hi[0] = hi.x; box.hi[1] = hi.y; box.hi[2] = hi.z;
                        box.r2 = gr * gr;
                        box.cx0 = max(CellMath<float>::coord(g, lo.x, 0) - extx, 0);
                        box.cx1 = min(CellMath<float>::coord(g, hi.x, 0) + extx, g.dim[0] - 1);
                        box.cy0 = max(CellMath<float>::coord(g, lo.y, 1) - ext, 0);
                        const int cy1 = min(CellMath<float>::coord(g, hi.y, 1) + ext, g.dim[1] - 1);
                        box.cz0 = max(CellMath<float>::coord(g, lo.z, 2) - ext, 0);
                        const int cz1 = min(CellMath<float>::coord(g, hi.z, 2) + ext, g.dim[2] - 1);
                        box.ny = cy1 - box.cy0 + 1;
                        box.nrows = box.ny * (cz1 - box.cz0 + 1);
                    }
                    __syncwarp();
                }
                const int nrows = box.nrows;
                for (int row0 = 0; row0 < nrows; row0 += 32) {
                    uint32_t rbeg = 0, rlen = 0;
                    const int row = row0 + (int)lane;
                    if (row < nrows) {
                        const int ny = box.ny;
                        const int zz = box.cz0 + row / ny, yy = box.cy0 + row % ny;
                        int x0, x1;
                        if (box_row_range(g, mk3(box.lo[0], box.lo[1], box.lo[2]), mk3(box.hi[0], box.hi[1], box.hi[2]),
                                          box.r2, yy, zz, box.cx0, box.cx1, x0, x1)) {
                            const int base = (zz * g.dim[1] + yy) * g.dim[0];
                            rbeg = start[base + x0];
                            rlen = start[base + x1 + 1] - rbeg;
                        }
                    }
                    uint32_t incl = rlen;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= (unsigned)o) incl += u;
                    }
                    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                    const uint32_t excl = incl - rlen;
                    // rows end to end; a lane's row by a 5-step search (the
                    // sweep over the staged batch below dwarfs it)
                    for (uint32_t b0 = 0; b0 < total; b0 += 32) {
                        const uint32_t j = b0 + lane;
                        int r = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1)
                            if (__shfl_sync(0xffffffffu, incl, r + step - 1) <= j) r += step;
                        const uint32_t rb = __shfl_sync(0xffffffffu, rbeg, r), rx = __shfl_sync(0xffffffffu, excl, r);
                        const bool v = j < total;
                        uint32_t wl = 3u;
                        float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pd = pa;
                        if (v) {
                            const uint32_t slot = rb + (j - rx);
                            const float4 p = __ldg(&smap[slot]);
                            const uint32_t m = __float_as_uint(p.w);
                            float inv;
                            const V3<float> d = oct_raw(m, inv);
                            pa = make_float4(p.x, p.y, p.z, 0.f);
                            pd = make_float4(-d.x * inv, -d.y * inv, -d.z * inv, 0.f);
                            wl = min(m >> 30, 2u);
                        }
                        const unsigned m0 = __ballot_sync(0xffffffffu, wl == 0u), m1 = __ballot_sync(0xffffffffu, wl == 1u),
                                       m2 = __ballot_sync(0xffffffffu, wl == 2u);
                        const int n0 = __popc(m0), n01 = n0 + __popc(m1), nv = n01 + __popc(m2);
                        if (v) {
                            const int at = wl == 0u ? __popc(m0 & lt) : (wl == 1u ? n0 + __popc(m1 & lt) : n01 + __popc(m2 & lt));
                            sp[at] = pa;
                            sd[at] = pd;
                        }
                        __syncwarp();
                        bool band = false;
                        auto sweep = [&](auto exact, int ta, int tb) -> uint32_t {
                            constexpr bool EXACT = decltype(exact)::value;
                            uint32_t acc = 0u;
#pragma unroll 2
                            for (int t = ta; t < tb; t++) {
                                const float4 a = sp[t], b = sd[t];
                                const float dx = q.x - a.x, dy = q.y - a.y, dz = q.z - a.z;
                                const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                                bool in = d2 < r2_lo;
                                const bool bd = !in && d2 <= r2_hi;
                                if constexpr (EXACT) {
                                    if (bd) in = sq_euclid(f2d_here(q.x), f2d_here(q.y), f2d_here(q.z), (double)a.x,
                                                           (double)a.y, (double)a.z) <= r2;
                                    if (COUNT && in) c_hits += 1;
                                } else {
                                    band |= bd;
                                }
                                const float c = __fmaf_rn(n.z, b.z, __fmaf_rn(n.y, b.y, n.x * b.x));
                                acc += fix_bits(in ? fmaxf(c, 0.0f) : 0.0f) - FIX_BIAS;
                            }
                            return acc;
                        };
                        uint32_t a0 = sweep(std::false_type{}, 0, n0);
                        uint32_t a1 = sweep(std::false_type{}, n0, n01);
                        uint32_t a2 = sweep(std::false_type{}, n01, nv);
                        if (__any_sync(0xffffffffu, band) || COUNT) {
                            a0 = sweep(std::true_type{}, 0, n0);
                            a1 = sweep(std::true_type{}, n0, n01);
                            a2 = sweep(std::true_type{}, n01, nv);
                        }
                        t0 += a0;
                        t1 += a1;
                        t2 += a2;
                        if (COUNT) {
                            c_tests += member ? (unsigned long long)nv : 0ull;
                            c_slots += (unsigned long long)nv;
                        }
                        __syncwarp();
                    }
                }
            }
        } else {
            // one query after another, the warp's lanes striding through its rows
            while (pending) {
                const int l = __ffs(pending) - 1;
                pending &= pending - 1;
                const float4 ql4 = s_own[wid][l];
                const V3<float> q = mk3(ql4.x, ql4.y, ql4.z);
                const V3<float> nl = mk3(__shfl_sync(0xffffffffu, n.x, l), __shfl_sync(0xffffffffu, n.y, l),
                                         __shfl_sync(0xffffffffu, n.z, l));
                const double r2l = __shfl_sync(0xffffffffu, r2, l);
                const float lo2 = __shfl_sync(0xffffffffu, r2_lo, l), hi2 = __shfl_sync(0xffffffffu, r2_hi, l);
                const float rl = ql4.w;
                const int ext = min(g.ext, max(1, (int)ceilf(rl * g.invf + 3e-3f)));
                const int extx = min(g.extx, max(1, (int)ceilf(rl * g.invxf + 3e-3f)));
                int c[3], lo[3], hi[3];
                query_cells(g, q, ext, extx, c, lo, hi);
                unsigned long long u0 = 0, u1 = 0, u2 = 0;
                // a lane adds at most one term (<= 2^23) per step: 32-bit lane
                // sums, folded into the 64-bit ones every 256 steps, cannot wrap
                uint32_t v0 = 0u, v1 = 0u, v2 = 0u, steps = 0u;
                // row by row: these rows already fill most lanes, and a packed
                // walk's lane placement costs more than it saves here
                for_each_candidate(g, start, q, rl * rl, lo, hi, [&](uint32_t idx, bool valid2) {
                    const float4 p = __ldg(&smap[idx]);
                    const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
                    const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                    bool in = valid2 && d2 < lo2;
                    const bool bd = valid2 && !in && d2 <= hi2;
                    if (__any_sync(0xffffffffu, bd))
                        if (bd) in = sq_euclid(f2d_here(q.x), f2d_here(q.y), f2d_here(q.z), (double)p.x, (double)p.y,
                                               (double)p.z) <= r2l;
                    if (in) {   // the term of a photon in radius (most candidates are not)
                        const uint32_t m = __float_as_uint(p.w);
                        float inv;
                        const V3<float> d = oct_raw(m, inv);
                        const float bx = -d.x * inv, by = -d.y * inv, bz = -d.z * inv;
                        const float cc = __fmaf_rn(nl.z, bz, __fmaf_rn(nl.y, by, nl.x * bx));
                        const uint32_t term = fix_bits(fmaxf(cc, 0.0f)) - FIX_BIAS;
                        const uint32_t w = m >> 30;
                        v0 += w == 0u ? term : 0u;
                        v1 += w == 1u ? term : 0u;
                        v2 += w >= 2u ? term : 0u;
                    }
                    if ((++steps & 255u) == 0u) {
                        u0 += v0; u1 += v1; u2 += v2;
                        v0 = v1 = v2 = 0u;
                    }
                    if (COUNT) {
                        c_slots += 1;
                        c_tests += valid2 ? 1 : 0;
                        c_hits += in ? 1 : 0;
                    }
                });
                u0 += v0; u1 += v1; u2 += v2;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    u0 += __shfl_xor_sync(0xffffffffu, u0, o);
                    u1 += __shfl_xor_sync(0xffffffffu, u1, o);
                    u2 += __shfl_xor_sync(0xffffffffu, u2, o);
                }
                if ((int)lane == l) { t0 = u0; t1 = u1; t2 = u2; }
            }
        }
        if (valid) {
            // the query's slot in the caller's arrays is its pixel field
            const int32_t dst = hits[qi].pixel;
            const double kk = FIX_UNIT * (pw * (ONE_PI_D / r2));
            double *o = out.out_rgb + 3 * (size_t)dst;
            o[0] = (double)t0 * kk;
            o[1] = (double)t1 * kk;
            o[2] = (double)t2 * kk;
        }
        __syncwarp();   // s_own is rewritten by the next chunk
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            c_tests += __shfl_xor_sync(0xffffffffu, c_tests, o);
            c_hits += __shfl_xor_sync(0xffffffffu, c_hits, o);
            c_slots += __shfl_xor_sync(0xffffffffu, c_slots, o);
        }
        if (lane == 0) {
            atomicAdd(out.count + 0, c_tests);
            atomicAdd(out.count + 1, c_hits);
            atomicAdd(out.count + 2, c_slots);
        }
    }
}

// Estimate queries are gathered in the map's cell order, so that the warps
// running at the same time walk the same cells and share photons in L2
// (random query order re-reads the map from HBM once per neighbourhood).
// k_query_hist ranks each query inside its cell (key 3*cell, the map's key
// space, so the map's scan sizes apply); k_query_place writes the hit point
// and its radius to the sorted slot, keeping the caller's index in pixel.
// The key's wavelength slot holds the query's radius class (r^2 below
// r2_a, below r2_b, the rest), so that inside a cell the queries are grouped
// by size: 32 consecutive queries then have similar radii, which is what
// lets k_estimate_tile share one walk among them.  Non-negative doubles
// order as their bit patterns, so the classes take integer compares.
__global__ void __launch_bounds__(256) k_query_hist(const float *pos, const double *r2, long long n,
                                                    const PassState *st, double r2_a, double r2_b, uint32_t *count,
                                                    uint2 *keyrank) {
    const GridParams g = st->grid;
    const long long ba = __double_as_longlong(r2_a), bb = __double_as_longlong(r2_b);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long br = __double_as_longlong(r2[i]);
        const uint32_t cls = br < ba ? 0u : (br < bb ? 1u : 2u);
        const uint32_t c = 3u * cell_of(g, ld3(pos + 3 * i)) + cls;
        keyrank[i] = make_uint2(c, atomicAdd(&count[c], 1u));
    }
}

__global__ void __launch_bounds__(256) k_query_place(const float *pos, const float *nrm, const double *r2, long long n,
                                                     const uint32_t *start, const uint2 *keyrank,
                                                     HitPoint<float> *hits, double *r2_sorted) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint2 kr = keyrank[i];
        const uint32_t dst = start[kr.x] + kr.y;
        HitPoint<float> h;
        for (int a = 0; a < 3; a++) { h.pos[a] = pos[3 * i + a]; h.nrm[a] = nrm[3 * i + a]; h.w[a] = 1.0f; }
        h.pixel = (int32_t)i;
        hits[dst] = h;
        r2_sorted[dst] = r2[i];
    }
}

#endif  // PPM_BUILD_F32

// ---------------------------------------------------------------------------
// in-radius sets (parity entry points): count pass, then fill pass
// ---------------------------------------------------------------------------
template <typename T, typename MapT>
__global__ void __launch_bounds__(256) k_within(const T *q, long long nq, const double *q_r2, const PassState *st,
                                                const MapT *smap, const uint32_t *start, const int32_t *sidx,
                                                unsigned long long *counts, const unsigned long long *offsets,
                                                int32_t *idx_out) {
    const GridParams g = st->grid;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long qi = warp; qi < (unsigned long long)nq; qi += nwarps) {
        V3<T> qq = ld3(q + 3 * qi);
        const double r2 = q_r2[qi];
        const float r2_lo = __double2float_rd(r2 * (1.0 - 1e-6));
        const float r2_hi = __double2float_ru(r2 * (1.0 + 1e-6));
        int ext = min(g.ext, max(1, (int)ceil(sqrt(r2) * g.inv + 3e-3)));
        int extx = min(g.extx, max(1, (int)ceil(sqrt(r2) * g.invx + 3e-3)));
        int c[3], lo[3], hi[3];
        query_cells(g, qq, ext, extx, c, lo, hi);
        unsigned long long found = 0;
        unsigned long long wbase = offsets ? offsets[qi] : 0;
        for_each_candidate(g, start, qq, (T)r2, lo, hi, [&](uint32_t idx, bool valid) {
            bool hit = false;
            int32_t orig = 0;
            if (valid) {
                if constexpr (sizeof(T) == 8) {
                    double4 pp = smap[idx];
                    hit = sq_euclid(qq.x, qq.y, qq.z, pp.x, pp.y, pp.z) <= r2;
                    orig = (int32_t)(((unsigned long long)__double_as_longlong(pp.w)) & 0xffffffffffULL);
                } else {
                    float d2f;
                    hit = in_radius_f32(qq.x, qq.y, qq.z, smap[idx], r2_lo, r2_hi, r2, d2f);
                    orig = sidx[idx];
                }
            }
            unsigned m = __ballot_sync(0xffffffffu, hit);
            if (idx_out && hit) idx_out[wbase + found + __popc(m & ((1u << lane_id()) - 1u))] = orig;
            found += __popc(m);
        });
        if (lane_id() == 0 && counts) counts[qi] = found;
    }
}

// queries from host arrays for the estimate entry points
template <typename T>
__global__ void k_make_queries(const T *pos, const T *nrm, long long n, HitPoint<T> *hits) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HitPoint<T> h;
    for (int a = 0; a < 3; a++) { h.pos[a] = pos[3 * i + a]; h.nrm[a] = nrm[3 * i + a]; h.w[a] = T(1); }
    h.pixel = (int32_t)i;
    hits[i] = h;
}

// first-hit parity kernel: calc_intersection for a batch of rays
template <typename T, bool B>
__global__ void k_intersect(SceneView<T, B> sc, const double *rays, long long n, double *t, int32_t *obj, double *nrm) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *r = rays + 6 * i;
    V3<T> rp = mk3((T)r[0], (T)r[1], (T)r[2]), rd = mk3((T)r[3], (T)r[4], (T)r[5]);
    Isect<T> is;
    if (intersect(sc, rp, rd, is)) {
        t[i] = (double)is.t; obj[i] = is.obj;
        if (nrm) { nrm[3 * i] = (double)is.n.x; nrm[3 * i + 1] = (double)is.n.y; nrm[3 * i + 2] = (double)is.n.z; }
    } else {
        t[i] = 0.0; obj[i] = -1;
        if (nrm) { nrm[3 * i] = 0.0; nrm[3 * i + 1] = 0.0; nrm[3 * i + 2] = 0.0; }
    }
}

// ---------------------------------------------------------------------------
// Batched passes: one launch per stage runs that stage for every job of a
// batch (k_batch.cu, and the per-job bookkeeping in k_grid.cu).  A job is a
// mixed-precision render with its own scene, camera, buffers and pass state;
// the stage kernels map their work items -- (job, element) -- onto the
// concatenation of the jobs' work, through a prefix of the jobs' counts.
// ---------------------------------------------------------------------------
constexpr int BATCH_MAX_JOBS = 256;   // the prefix of job counts lives in one block's shared memory

struct JobDev {
    SceneView<float> sv;          // bvh != nullptr: rays walk the hierarchy
    DCamera<float> cam;
    EmitPlan plan;
    PassState *st;
    uint64_t seed;
    float4 *raw, *sorted;         // stored photons and the photon map
    uint32_t *count, *start, *block_sums;
    uint2 *keyrank;
    HitPoint<float> *hits;
    EyeQueue<float> qa, qb;
    unsigned long long eq_cap;
    float *direct, *gathered;
    double *pass_img, *sum_img;
    double pw;
    long long npx;
    int32_t uc, pfilter;
};

// counters the stages take their work from (reset by the batch's first stage)
struct BatchState {
    unsigned long long emit_next, gather_next;
};

// prefix[j] = sum of count(k) for k < j, prefix[njobs] = total, in shared
// memory; the block's threads (at least njobs of them) load one count each
template <typename F>
__device__ __forceinline__ long long batch_prefix(long long *prefix, int njobs, F count) {
    __shared__ long long wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    long long v = t < njobs ? count(t) : 0;
    long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    long long before = 0;
    for (int k = 0; k < w; k++) before += wsum[k];
    if (t < njobs) prefix[t] = before + incl - v;
    if (t == (int)blockDim.x - 1) prefix[njobs] = before + incl;
    __syncthreads();
    return prefix[njobs];
}

// the job of flattened index x: the last j with prefix[j] <= x
__device__ __forceinline__ int batch_job(const long long *prefix, int njobs, long long x) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace ppm
