// ppm_api.cu -- host runtime behind include/ppm_api.h.
//
// A context owns one CUDA stream (plus a side stream that runs the eye pass
// concurrently with photon tracing), all device buffers and the device-side
// PassState.  One progressive pass is a fixed sequence of kernels whose
// parameters live in device memory, so it is captured once as a CUDA graph
// and replayed for every pass.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ppm_api.h"
#include "ppm_launch.h"

using namespace ppm;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// stages 0-4 are timed per render pass; map_build, gather and query_sort are
// also timed by the FP32 map entry points (photon map build, estimate)
constexpr int N_RENDER_STAGES = 5;
constexpr int N_STAGES = 6;
const char *STAGE_NAMES[N_STAGES] = {"photon_trace", "map_build", "eye_trace", "gather", "accumulate", "query_sort"};
constexpr int TIMING_SLOTS = 256;
constexpr int HITS_PER_PIXEL = 8;
constexpr long long CELL_CAP = 1LL << 24;   // map keys (one per cell), the most one scan takes
constexpr int BVH_MIN_OBJECTS = 32;   // below this a loop over the objects is faster
constexpr int MAX_CELL_FACTOR = 4;    // render grids: 1 to 4 cells per radius (the tuner tries each)

thread_local std::string g_create_error;

}  // namespace

struct ppm_ctx {
    int device = 0;
    int sm_count = 0;
    int tile_blocks = 1;   // resident blocks per SM of the render's tile gather
    int est_blocks = 1;    // and of the estimate entry point's chunk gather
    cudaStream_t s = nullptr, s2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string err;
    // every object bounded: the box the render's grids span (set at upload);
    // render_scene_box: the begun render uses it
    bool scene_box = false, render_scene_box = false;
    double scene_lo[3] = {0, 0, 0}, scene_hi[3] = {0, 0, 0};
    uint64_t seed = 0;

    // scene
    std::vector<ppm_object> objs;
    std::vector<ppm_material> mats;
    std::vector<ppm_light> lights;
    DevBuf objs_d, mats_d, lights_d, objs_f, mats_f, lights_f;
    DevBuf bvh_nodes, bvh_bounded, bvh_unb, bvh_order;   // hierarchy over the bounded objects
    int accel_mode = 0;                        // PPM_ACCEL_*
    int bvh_leaf = 1;                          // objects per leaf (1..8)
    int bvh_m = 0;                             // objects in the hierarchy (0: none)
    SceneView<double> sv_d{};
    SceneView<float> sv_f{};
    const SceneView<double> &sv_of(double) const { return sv_d; }
    const SceneView<float> &sv_of(float) const { return sv_f; }
    bool have_scene = false;
    ppm_camera cam{};
    DCamera<double> cam_d{};
    DCamera<float> cam_f{};
    bool have_cam = false;

    // device state and buffers
    PassState *st = nullptr;
    DevBuf raw_d, spos, sdir, raw_f, sorted_f, sidx, keyrank, count, start, block_sums;
    long long photon_cap_d = 0, photon_cap_f = 0;
    DevBuf eqb[6];                // eye queues: A(a, b, c), B(a, b, c)
    long long eq_cap = 0;
    DevBuf hits_d, hits_f;
    long long hit_cap = 0;
    DevBuf pass_img, sum_img;
    DevBuf pass_direct32, pass_gather32;   // FP32 path per-pass buffers
    DevBuf gdump;                          // render gather parity export records
    // the mixed render's hit points in Morton order (the gathers' input):
    // sorted copy, key/rank per hit point, key counts, starts, scan tile sums
    DevBuf hits_sorted, hkeyrank, hcount, hstart, hblock;
    DevBuf tile_queue;                     // the tile gather's queue of split walks
    unsigned long long tile_cap = 0;       // its entries
    GatherDump *gather_dump = nullptr;     // set while the export pass is enqueued
    long long npx = 0;
    DevBuf scratch;   // parity entry-point staging
    DevBuf qstart;    // estimate queries: cell starts of the query sort
    char *noalloc_base = nullptr;   // device address of the allocation-free estimate's array on this device

    // parity photon map
    int map_kind = 0;  // 0 none, 1 f64, 2 f32
    long long map_n = 0;
    double map_pw = 0.0, map_r2 = 0.0;
    double map_cells = 2.0;   // FP32 map: grid cells per maximum query radius
    int last_trace_uc = 1;
    double last_trace_pw = 0.0;

    // render
    ppm_render_cfg cfg{};
    bool render_ready = false;
    EmitPlan plan{};
    double pw = 0.0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    long long passes_done = 0;
    int kernels_per_pass = 0;
    int cell_factor = 0;          // grid cells per radius of the current render
    // x cells per y/z cell of the render's photon map: 4 measured best on the
    // glass box (gather 0.586 -> 0.526 ms) and the mesh (17.3 -> 15.5 ms)
    // against 1, 2 and 8
    int render_sx = 4;

    // timing
    bool timing = false;
    bool count_gather = false;
    cudaEvent_t tev[TIMING_SLOTS][8];
    bool tev_made = false;
    cudaEvent_t xev[4];   // FP32 map entry points: build / sort / gather brackets
    int slot_head = 0, slot_pending = 0;
    double stage_ms[16] = {0};
    long long stage_calls[16] = {0};
};

static int set_err(ppm_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return set_err(ctx, e_ == cudaErrorMemoryAllocation ? PPM_ERR_OOM : PPM_ERR_CUDA,     \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

static int ensure(ppm_ctx *ctx, DevBuf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return PPM_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    CK(cudaMalloc(&b.p, bytes));
    b.bytes = bytes;
    return PPM_OK;
}

static void release(DevBuf &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

template <typename T> static T *as(DevBuf &b) { return static_cast<T *>(b.p); }

#define CK_B(call)                                                                                 \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return batch_err(b, PPM_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
    } while (0)

#define TRY(x)                          \
    do {                                \
        int r_ = (x);                   \
        if (r_ != PPM_OK) return r_;    \
    } while (0)

// ---------------------------------------------------------------------------
// host-side derivations (same formulas and evaluation order as the reference)
// ---------------------------------------------------------------------------
namespace {
struct HV {
    double x, y, z;
};
HV hv(const double *p) { return {p[0], p[1], p[2]}; }
HV hadd(HV a, HV b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
HV hsub(HV a, HV b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
HV hsm(double s, HV a) { return {s * a.x, s * a.y, s * a.z}; }
double hdot(HV a, HV b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HV hcross(HV a, HV b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
HV hnorm(HV a) {
    double n = std::sqrt(hdot(a, a));
    if (n == 0.0) return a;
    double r = 1.0 / n;
    return {a.x * r, a.y * r, a.z * r};
}
void hst(double *d, HV v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }
}  // namespace

extern "C" void ppm_camera_derive(ppm_camera *c) {
    // camera.rs:150-175
    const double SENSOR = 35.0 / 1000.0, ISO = 100.0, FNUM = 4.9, SHUT = 1.0 / 250.0;
    HV eye = hv(c->eye_pos), tgt = hv(c->target), up = hv(c->upper);
    HV ez = hnorm(hsub(tgt, eye));
    HV ex = hnorm(hcross(up, ez));
    HV ey = hnorm(hcross(ex, ez));
    double step = (c->focus * SENSOR / c->focal_len) / (double)c->xreso;
    HV esx = hsm(step, ex), esy = hsm(step, ey);
    double ea = c->focal_len / c->f_number;
    HV eex = hsm(ea, ex), eey = hsm(ea, ey);
    double lx = (double)(c->xreso / 2), ly = (double)(c->yreso / 2);
    HV orig = hsub(hsub(hsm(c->focus, ez), hsm(lx - 0.5, esx)), hsm(ly - 0.5, esy));
    c->photon_power = c->blur ? c->iso_sens / ISO * FNUM / c->f_number * c->shut_speed / SHUT : 1.0;
    hst(c->eye_dir, hnorm(hsub(tgt, eye)));
    hst(c->origin, orig);
    hst(c->esx, esx);
    hst(c->esy, esy);
    hst(c->eex, eex);
    hst(c->eey, eey);
}

extern "C" void ppm_material_derive(ppm_material *m) {
    // Surface::new_simple / new_ts, surface.rs:52 and :63-64
    m->density_pow = 1.0 / (std::pow(10.0, 5.0 * (1.0 - std::sqrt(m->roughness))) + 1.0);
    double r = m->roughness;
    m->alpha = m->surface == PPM_SURF_TS ? r * r * r * r : 0.0;
}

// ---------------------------------------------------------------------------
// scene conversion
// ---------------------------------------------------------------------------
template <typename T>
static void conv_objects(const std::vector<ppm_object> &in, std::vector<DObject<T>> &out) {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); i++) {
        const ppm_object &o = in[i];
        DObject<T> &d = out[i];
        d.shape = o.shape;
        d.mat = o.material;
        for (int a = 0; a < 3; a++) {
            d.p[a] = (T)o.position[a];
            d.n[a] = (T)o.nvec[a];
            d.d1[a] = (T)o.dir1[a];
            d.d2[a] = (T)o.dir2[a];
        }
        d.dist = (T)o.dist;
        d.radius = (T)o.radius;
    }
}

static uint32_t mat_flags(const ppm_material &m) {
    auto eq = [](const double *c, double v) { return c[0] == v && c[1] == v && c[2] == v; };
    uint32_t f = 0;
    if (eq(m.color_spec, 0.0)) f |= 1u;
    if (eq(m.color_spec, 1.0)) f |= 2u;
    if (eq(m.color_diff, 0.0)) f |= 4u;
    return f;
}

template <typename T>
static void conv_materials(const std::vector<ppm_material> &in, std::vector<DMaterial<T>> &out) {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); i++) {
        const ppm_material &m = in[i];
        DMaterial<T> &d = out[i];
        for (int a = 0; a < 3; a++) {
            d.emit[a] = (T)m.emittance[a];
            d.ior[a] = (T)m.ior[a];
            d.cdiff[a] = (T)m.color_diff[a];
            d.cspec[a] = (T)m.color_spec[a];
        }
        d.scatter = (T)m.scatter;
        d.metal = (T)m.metalness;
        d.rough = (T)m.roughness;
        d.dpow = (T)m.density_pow;
        d.surface = m.surface;
        d.flags = mat_flags(m);
    }
}

template <typename T>
static void conv_lights(const std::vector<ppm_light> &in, std::vector<DLight<T>> &out) {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); i++) {
        const ppm_light &l = in[i];
        DLight<T> &d = out[i];
        d.kind = l.kind;
        d.pad = 0;
        for (int a = 0; a < 3; a++) {
            d.color[a] = (T)l.color[a];
            d.pos[a] = (T)l.pos[a];
            d.nvec[a] = (T)l.nvec[a];
            d.d1[a] = (T)l.dir1[a];
            d.d2[a] = (T)l.dir2[a];
            d.dir[a] = (T)l.dir[a];
        }
        d.flux = (T)l.flux;
    }
}

template <typename T>
static void conv_camera(const ppm_camera &c, DCamera<T> &d) {
    for (int a = 0; a < 3; a++) {
        d.eye[a] = (T)c.eye_pos[a];
        d.origin[a] = (T)c.origin[a];
        d.esx[a] = (T)c.esx[a];
        d.esy[a] = (T)c.esy[a];
        d.eex[a] = (T)c.eex[a];
        d.eey[a] = (T)c.eey[a];
        d.ambient[a] = (T)c.ambient[a];
    }
    d.xreso = c.xreso;
    d.yreso = c.yreso;
    d.jitter_aa = (c.progressive && c.antialias) ? 1 : 0;
    d.blur = c.blur ? 1 : 0;
}

template <typename V>
static int upload_vec(ppm_ctx *ctx, DevBuf &b, const std::vector<V> &v) {
    TRY(ensure(ctx, b, sizeof(V) * (v.size() ? v.size() : 1)));
    if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice, ctx->s));
    return PPM_OK;
}

// emission plan: ppmpa.rs:30-31 (pw = sum flux / N; n_l = round(flux_l / pw))
static double make_plan(const std::vector<ppm_light> &lights, long long nphoton, EmitPlan &plan) {
    double total = 0.0;
    for (const auto &l : lights) total = total + l.flux;
    double pw = total / (double)nphoton;
    plan.n_lights = (int32_t)lights.size();
    plan.first[0] = 0;
    for (size_t i = 0; i < lights.size(); i++) plan.first[i + 1] = plan.first[i] + (int64_t)std::llround(lights[i].flux / pw);
    return pw;
}

// The box of the scene's objects, when every object that can be hit is
// bounded (spheres, triangles, parallelograms; a point object is never hit):
// the render's photons and hit points lie on them, so its grids span this
// box without a bounds pass.  An infinite plane leaves scene_box false.
static void scene_bounds(ppm_ctx *ctx) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    bool ok = false;
    auto add = [&](const double *p, double dx, double dy, double dz) {
        const double v[3] = {p[0] + dx, p[1] + dy, p[2] + dz};
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], v[a]);
            hi[a] = std::max(hi[a], v[a]);
        }
    };
    for (const ppm_object &o : ctx->objs) {
        const double *p = o.position, *d1 = o.dir1, *d2 = o.dir2;
        switch (o.shape) {
        case SH_SPHERE:
            add(p, -o.radius, -o.radius, -o.radius);
            add(p, o.radius, o.radius, o.radius);
            ok = true;
            break;
        case SH_POLYGON:
        case SH_PARALLELOGRAM:
            add(p, 0.0, 0.0, 0.0);
            add(p, d1[0], d1[1], d1[2]);
            add(p, d2[0], d2[1], d2[2]);
            if (o.shape == SH_PARALLELOGRAM) add(p, d1[0] + d2[0], d1[1] + d2[1], d1[2] + d2[2]);
            ok = true;
            break;
        case SH_PLAIN:
            ctx->scene_box = false;
            return;
        default:
            break;
        }
    }
    bool finite = ok;
    for (int a = 0; a < 3; a++) finite = finite && lo[a] <= hi[a] && hi[a] - lo[a] < 1e30;
    ctx->scene_box = finite;
    for (int a = 0; a < 3; a++) {
        ctx->scene_lo[a] = finite ? lo[a] : 0.0;
        ctx->scene_hi[a] = finite ? hi[a] : 0.0;
    }
}

// cell_cap: cells a grid may have (map keys are cells; the FP32 estimate
// maps pass CELL_CAP / 3, so that their query sort's three radius classes
// per cell fit one scan)
static int upload_state(ppm_ctx *ctx, double r2, int pass, double alpha, int offset, double cell_factor,
                        long long photon_cap, long long hit_cap, int cell_sx = 1, long long cell_cap = CELL_CAP,
                        bool use_scene_box = false) {
    PassState h;
    std::memset(&h, 0, sizeof h);
    h.photon_cap = (unsigned long long)photon_cap;
    h.hit_cap = (unsigned long long)hit_cap;
    h.r2 = r2;
    h.alpha = alpha;
    h.pass = pass;
    h.offset = offset;
    h.cell_factor = cell_factor;
    h.cell_sx = cell_sx;
    h.cell_cap = cell_cap;
    h.scene_box = use_scene_box && ctx->scene_box ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        h.scene_lo[a] = ctx->scene_lo[a];
        h.scene_hi[a] = ctx->scene_hi[a];
    }
    CK(cudaMemcpyAsync(ctx->st, &h, sizeof h, cudaMemcpyHostToDevice, ctx->s));
    return PPM_OK;
}

static int read_state(ppm_ctx *ctx, PassState &h) {
    CK(cudaMemcpyAsync(&h, ctx->st, sizeof h, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PPM_OK;
}

static int add_stage_time(ppm_ctx *ctx, int stage, cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, a, b));
    ctx->stage_ms[stage] += ms;
    ctx->stage_calls[stage] += 1;
    return PPM_OK;
}

static int ensure_grid(ppm_ctx *ctx) {
    if (ctx->count.bytes == 0) {
        TRY(ensure(ctx, ctx->count, sizeof(uint32_t) * CELL_CAP));
        CK(cudaMemsetAsync(ctx->count.p, 0, sizeof(uint32_t) * CELL_CAP, ctx->s));
    }
    TRY(ensure(ctx, ctx->start, sizeof(uint32_t) * (CELL_CAP + 1)));
    TRY(ensure(ctx, ctx->block_sums, sizeof(uint32_t) * (CELL_CAP / SCAN_TILE + 1)));
    return PPM_OK;
}

static int grid_blocks(ppm_ctx *ctx, int per_sm) { return ctx->sm_count * per_sm; }

// buffers of the mixed render's hit point sort (hit_cap must be set); the key
// counts start zeroed and every scan leaves them zeroed
static int ensure_hit_sort(ppm_ctx *ctx) {
    TRY(ensure(ctx, ctx->hits_sorted, sizeof(HitPoint<float>) * (size_t)ctx->hit_cap));
    TRY(ensure(ctx, ctx->hkeyrank, sizeof(uint2) * (size_t)ctx->hit_cap));
    if (ctx->hcount.bytes == 0) {
        TRY(ensure(ctx, ctx->hcount, sizeof(uint32_t) * HIT_KEYS));
        CK(cudaMemsetAsync(ctx->hcount.p, 0, sizeof(uint32_t) * HIT_KEYS, ctx->s));
    }
    TRY(ensure(ctx, ctx->hstart, sizeof(uint32_t) * (HIT_KEYS + 1)));
    TRY(ensure(ctx, ctx->hblock, sizeof(uint32_t) * (HIT_KEYS / SCAN_TILE + 1)));
    // split walks: up to 8 per chunk of 32 hit points (a full queue only
    // means the warps walk the rest themselves)
    ctx->tile_cap = std::max(1024ULL, (unsigned long long)ctx->hit_cap / 4);
    TRY(ensure(ctx, ctx->tile_queue, sizeof(TileItem) * (size_t)ctx->tile_cap));
    return PPM_OK;
}

constexpr int EYE_QUEUE_PER_PIXEL = 2;   // eye-tree vertices per pixel a level may hold

static int ensure_eye_queues(ppm_ctx *ctx, long long npx, size_t vec_bytes) {
    long long cap = std::max(1LL, npx * EYE_QUEUE_PER_PIXEL);
    for (DevBuf &b : ctx->eqb) TRY(ensure(ctx, b, vec_bytes * (size_t)cap));
    ctx->eq_cap = cap;
    return PPM_OK;
}

// the persistent photon trace of one pass, in the precision of the photon buffer
static void launch_trace(ppm_ctx *ctx, const EmitPlan &plan, uint64_t seed, int uc, PhotonBuf<double> pb, int g,
                         cudaStream_t s) {
    launch_trace_d(ctx->sv_d, plan, seed, ctx->st, uc, pb, g, s);
}
static void launch_trace(ppm_ctx *ctx, const EmitPlan &plan, uint64_t seed, int uc, PhotonBuf<float> pb, int g,
                         cudaStream_t s) {
    launch_trace_f(ctx->sv_f, plan, seed, ctx->st, uc, pb, g, s);
}

// Eye levels after the first beside the photon trace: FP32 box scenes (no
// hierarchy; the classic tracer has no photon trace).  The trace then leaves
// room for one eye block per SM, so the levels run while it does instead of
// after it (the levels are latency-bound: each is a few dependent memory
// round trips long, whatever its size).
static bool eye_beside_trace(const ppm_ctx *ctx, bool fp32) {
    return fp32 && !ctx->sv_f.bvh && !(ctx->cfg.flags & PPM_RENDER_CLASSIC);
}

// one persistent launch with as many blocks as stay resident (TraceBlocks),
// or TRACE_BLOCKS_BESIDE_EYE per SM beside the eye levels
template <typename T>
static int enqueue_photon_trace(ppm_ctx *ctx, const EmitPlan &plan, uint64_t seed, int uc, PhotonBuf<T> pb,
                                cudaStream_t s) {
    const int per_sm = eye_beside_trace(ctx, sizeof(T) == 4) ? TRACE_BLOCKS_BESIDE_EYE : TraceBlocks<T>::value;
    launch_trace(ctx, plan, seed, uc, pb, grid_blocks(ctx, per_sm), s);
    return 1;
}

template <typename T, typename Level>
static int enqueue_eye(ppm_ctx *ctx, HitPoint<T> *hits, Level level_fn, cudaStream_t s) {
    using V = vec4_t<T>;
    EyeQueue<T> qa{as<V>(ctx->eqb[0]), as<V>(ctx->eqb[1]), as<V>(ctx->eqb[2])};
    EyeQueue<T> qb{as<V>(ctx->eqb[3]), as<V>(ctx->eqb[4]), as<V>(ctx->eqb[5])};
    // Level 0 has one thread per pixel slot (pixels in tiles of 32, see
    // eye_slots), striding over them.  Beside the photon trace its grid is
    // two blocks per SM, so the trace's blocks start at once on the rest
    // of each SM instead of waiting for a wave of sixteen eye blocks to
    // drain.  The deeper levels' sizes are only known on the device; their
    // grids stride over the queue: two blocks per SM beside the trace (one
    // runs in the room the trace leaves, the other once it ends), four
    // otherwise.
    const bool beside = eye_beside_trace(ctx, sizeof(T) == 4);
    const long long slots = eye_slots(ctx->cam.xreso, ctx->cam.yreso);
    const long long g0_cap = (long long)ctx->sm_count * (beside ? 2 : 16);
    const int g0 = (int)std::max(1LL, std::min<long long>((slots + 127) / 128, g0_cap));
    const int gl = grid_blocks(ctx, beside ? 2 : 4);
    for (int l = 0; l < MAX_TRACE; l++)
        level_fn(l, (l & 1) ? qb : qa, (l & 1) ? qa : qb, (unsigned long long)ctx->eq_cap, hits, l == 0 ? g0 : gl,
                 s);
    return MAX_TRACE;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" int ppm_version(void) { return PPM_API_VERSION; }

extern "C" const char *ppm_status_string(int s) {
    switch (s) {
    case PPM_OK: return "ok";
    case PPM_ERR_INVALID_ARG: return "invalid argument";
    case PPM_ERR_OOM: return "out of device memory";
    case PPM_ERR_CAPACITY: return "capacity exceeded";
    case PPM_ERR_TIMEOUT: return "timeout";
    case PPM_ERR_CUDA: return "CUDA error";
    case PPM_ERR_NOT_READY: return "not ready";
    case PPM_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

static cudaError_t noalloc_lookup(char **out);

// The eye pass runs on a side stream beside the photon trace; it gets the
// higher priority, so its blocks are scheduled first when both wait.
static int eye_priority() {
    int lo = 0, hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) return 0;
    return hi;
}

extern "C" int ppm_ctx_create(ppm_ctx **out, int device, uint64_t seed) {
    if (!out) return PPM_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0 || device < 0 || device >= n) {
        g_create_error = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count 0 or bad index");
        return PPM_ERR_NO_DEVICE;
    }
    ppm_ctx *ctx = new ppm_ctx();
    ctx->device = device;
    ctx->seed = seed;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete ctx;
        return PPM_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    ctx->tile_blocks = gather_tile_blocks_per_sm();
    ctx->est_blocks = estimate_tile_blocks_per_sm();
    if (cudaStreamCreateWithFlags(&ctx->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->s2, cudaStreamNonBlocking, eye_priority()) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&ctx->st, sizeof(PassState)) != cudaSuccess) {
        g_create_error = "stream/event/state allocation failed";
        ppm_ctx_destroy(ctx);
        return PPM_ERR_CUDA;
    }
    // the allocation-free estimate's array and kernels: placed on the device
    // and its address resolved now, so that ppm_estimate_noalloc never loads
    // or allocates anything
    cudaError_t ea = noalloc_lookup(&ctx->noalloc_base);
    if (ea == cudaSuccess) ea = load_estimate_kernels_d();
    if (ea != cudaSuccess) {
        g_create_error = std::string("placing the allocation-free estimate's array and kernels: ") + cudaGetErrorString(ea);
        ppm_ctx_destroy(ctx);
        return PPM_ERR_CUDA;
    }
    *out = ctx;
    return PPM_OK;
}

static void drop_graph(ppm_ctx *ctx) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->graph_exec = nullptr;
    ctx->graph = nullptr;
}

extern "C" int ppm_ctx_destroy(ppm_ctx *ctx) {
    if (!ctx) return PPM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->s) cudaStreamSynchronize(ctx->s);
    if (ctx->s2) cudaStreamSynchronize(ctx->s2);
    drop_graph(ctx);
    DevBuf *bufs[] = {&ctx->objs_d, &ctx->mats_d, &ctx->lights_d, &ctx->objs_f, &ctx->mats_f, &ctx->lights_f,
                      &ctx->raw_d, &ctx->spos, &ctx->sdir, &ctx->raw_f, &ctx->sorted_f, &ctx->sidx,
                      &ctx->keyrank, &ctx->count, &ctx->start, &ctx->block_sums, &ctx->hits_d, &ctx->hits_f,
                      &ctx->pass_img, &ctx->sum_img, &ctx->scratch, &ctx->pass_direct32, &ctx->pass_gather32,
                      &ctx->qstart, &ctx->bvh_nodes, &ctx->bvh_bounded, &ctx->bvh_unb, &ctx->bvh_order,
                      &ctx->gdump, &ctx->hits_sorted, &ctx->hkeyrank, &ctx->hcount, &ctx->hstart, &ctx->hblock,
                      &ctx->tile_queue};
    for (DevBuf *b : bufs) release(*b);
    for (DevBuf &b : ctx->eqb) release(b);
    if (ctx->st) cudaFree(ctx->st);
    if (ctx->tev_made) {
        for (int i = 0; i < TIMING_SLOTS; i++)
            for (int j = 0; j < 8; j++) cudaEventDestroy(ctx->tev[i][j]);
        for (cudaEvent_t e : ctx->xev) cudaEventDestroy(e);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->s) cudaStreamDestroy(ctx->s);
    if (ctx->s2) cudaStreamDestroy(ctx->s2);
    delete ctx;
    return PPM_OK;
}

extern "C" const char *ppm_last_error(const ppm_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }
extern "C" void *ppm_ctx_stream(ppm_ctx *ctx) { return ctx ? (void *)ctx->s : nullptr; }
extern "C" int ppm_ctx_sync(ppm_ctx *ctx) {
    if (!ctx) return PPM_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(ctx->s));
    CK(cudaStreamSynchronize(ctx->s2));
    return PPM_OK;
}

// ---------------------------------------------------------------------------
// scene and camera
// ---------------------------------------------------------------------------
// Objects reached through the hierarchy: spheres, triangles, parallelograms.
// Infinite planes are tested on every ray; points are never hit.
static bool bounded_shape(int shape) {
    return shape == PPM_SHAPE_SPHERE || shape == PPM_SHAPE_POLYGON || shape == PPM_SHAPE_PARALLELOGRAM;
}

static int build_accel(ppm_ctx *ctx) {
    std::vector<int32_t> bounded, unb;
    for (int i = 0; i < (int)ctx->objs.size(); i++) {
        if (bounded_shape(ctx->objs[i].shape)) bounded.push_back(i);
        else if (ctx->objs[i].shape == PPM_SHAPE_PLAIN) unb.push_back(i);
    }
    const int m = (int)bounded.size();
    const bool use = ctx->accel_mode == PPM_ACCEL_BVH ? m >= 2
                   : ctx->accel_mode == PPM_ACCEL_NONE ? false : m >= BVH_MIN_OBJECTS;
    for (auto *v : {&ctx->sv_d}) { v->bvh = nullptr; v->bvh_order = nullptr; v->unb = nullptr; v->n_unb = 0; v->bvh_root = 0; v->bvh_steps = 0; }
    for (auto *v : {&ctx->sv_f}) { v->bvh = nullptr; v->bvh_order = nullptr; v->unb = nullptr; v->n_unb = 0; v->bvh_root = 0; v->bvh_steps = 0; }
    ctx->bvh_m = 0;
    if (!use) return PPM_OK;
    if (m > (1 << 28)) return set_err(ctx, PPM_ERR_INVALID_ARG, "at most 2^28 bounded objects");
    TRY(upload_vec(ctx, ctx->bvh_bounded, bounded));
    if (!unb.empty()) TRY(upload_vec(ctx, ctx->bvh_unb, unb));
    TRY(ensure(ctx, ctx->bvh_nodes, sizeof(BvhNode) * (size_t)(m - 1)));
    TRY(ensure(ctx, ctx->bvh_order, sizeof(int32_t) * (size_t)m));
    DevBuf scratch;
    const int n_objs = (int)ctx->objs.size();
    if (cudaMalloc(&scratch.p, sizeof(uint32_t) * (size_t)bvh_scratch_words(m, n_objs)) != cudaSuccess)
        return set_err(ctx, PPM_ERR_OOM, "no device memory for the BVH build of %d objects", m);
    const int root = launch_bvh_build(as<DObject<double>>(ctx->objs_d), as<int32_t>(ctx->bvh_bounded), m, n_objs,
                                      ctx->bvh_leaf,
                                      as<BvhNode>(ctx->bvh_nodes), as<int32_t>(ctx->bvh_order), as<uint32_t>(scratch),
                                      ctx->s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->s);
    cudaFree(scratch.p);
    if (e != cudaSuccess) return set_err(ctx, PPM_ERR_CUDA, "BVH build: %s", cudaGetErrorString(e));
    const BvhNode *nodes = as<BvhNode>(ctx->bvh_nodes);
    const int32_t *u = unb.empty() ? nullptr : as<int32_t>(ctx->bvh_unb);
    const int32_t steps = 2 * m + 64;
    const int32_t *order = as<int32_t>(ctx->bvh_order);
    ctx->sv_d.bvh = nodes; ctx->sv_d.unb = u; ctx->sv_d.n_unb = (int32_t)unb.size(); ctx->sv_d.bvh_steps = steps;
    ctx->sv_f.bvh = nodes; ctx->sv_f.unb = u; ctx->sv_f.n_unb = (int32_t)unb.size(); ctx->sv_f.bvh_steps = steps;
    ctx->sv_d.bvh_order = order; ctx->sv_f.bvh_order = order;
    ctx->sv_d.bvh_root = root; ctx->sv_f.bvh_root = root;
    ctx->sv_d.bvh_runs = ctx->sv_f.bvh_runs = ctx->bvh_leaf > 1 ? 1 : 0;
    ctx->bvh_m = m;
    return PPM_OK;
}

extern "C" int ppm_scene_upload(ppm_ctx *ctx, const ppm_object *objs, int32_t n_objs, const ppm_material *mats,
                                int32_t n_mats, const ppm_light *lights, int32_t n_lights) {
    if (!ctx) return PPM_ERR_INVALID_ARG;
    if (n_objs < 0 || n_mats < 0 || n_lights < 0 || n_lights > 16 || (n_objs && !objs) || (n_mats && !mats) ||
        (n_lights && !lights))
        return set_err(ctx, PPM_ERR_INVALID_ARG, "bad scene arrays (n_objs=%d n_mats=%d n_lights=%d, at most 16 lights)",
                       n_objs, n_mats, n_lights);
    for (int i = 0; i < n_objs; i++)
        if (objs[i].material < 0 || objs[i].material >= n_mats || objs[i].shape < 0 || objs[i].shape > 4)
            return set_err(ctx, PPM_ERR_INVALID_ARG, "object %d: bad material index %d or shape %d", i,
                           objs[i].material, objs[i].shape);
    for (int i = 0; i < n_lights; i++) {
        if (lights[i].kind < 0 || lights[i].kind > PPM_LIGHT_SPOT)
            return set_err(ctx, PPM_ERR_INVALID_ARG, "light %d: bad kind %d", i, lights[i].kind);
        if (lights[i].kind == PPM_LIGHT_SPOT && !(lights[i].dir1[0] >= -1.0 && lights[i].dir1[0] <= 1.0))
            return set_err(ctx, PPM_ERR_INVALID_ARG, "light %d: spot cos(half-angle) %g outside [-1, 1]", i,
                           lights[i].dir1[0]);
    }
    cudaSetDevice(ctx->device);
    ctx->objs.assign(objs, objs + n_objs);
    ctx->mats.assign(mats, mats + n_mats);
    ctx->lights.assign(lights, lights + n_lights);
    scene_bounds(ctx);
    std::vector<DObject<double>> od;
    std::vector<DObject<float>> of;
    std::vector<DMaterial<double>> md;
    std::vector<DMaterial<float>> mf;
    std::vector<DLight<double>> ld;
    std::vector<DLight<float>> lf;
    conv_objects(ctx->objs, od);
    conv_objects(ctx->objs, of);
    conv_materials(ctx->mats, md);
    conv_materials(ctx->mats, mf);
    conv_lights(ctx->lights, ld);
    conv_lights(ctx->lights, lf);
    TRY(upload_vec(ctx, ctx->objs_d, od));
    TRY(upload_vec(ctx, ctx->objs_f, of));
    TRY(upload_vec(ctx, ctx->mats_d, md));
    TRY(upload_vec(ctx, ctx->mats_f, mf));
    TRY(upload_vec(ctx, ctx->lights_d, ld));
    TRY(upload_vec(ctx, ctx->lights_f, lf));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->sv_d = SceneView<double>{as<DObject<double>>(ctx->objs_d), as<DMaterial<double>>(ctx->mats_d),
                                  as<DLight<double>>(ctx->lights_d), n_objs, n_mats, n_lights, 0, nullptr, nullptr, 0, 0};
    ctx->sv_f = SceneView<float>{as<DObject<float>>(ctx->objs_f), as<DMaterial<float>>(ctx->mats_f),
                                 as<DLight<float>>(ctx->lights_f), n_objs, n_mats, n_lights, 0, nullptr, nullptr, 0, 0};
    ctx->have_scene = true;
    ctx->render_ready = false;
    drop_graph(ctx);
    return build_accel(ctx);
}

extern "C" int ppm_set_accel(ppm_ctx *ctx, int32_t mode) {
    if (!ctx || mode < PPM_ACCEL_AUTO || mode > PPM_ACCEL_NONE) return PPM_ERR_INVALID_ARG;
    ctx->accel_mode = mode;
    if (!ctx->have_scene) return PPM_OK;
    cudaSetDevice(ctx->device);
    ctx->render_ready = false;
    drop_graph(ctx);
    return build_accel(ctx);
}

extern "C" int ppm_set_bvh_leaf(ppm_ctx *ctx, int32_t leaf_max) {
    if (!ctx || leaf_max < 1 || leaf_max > 8) return PPM_ERR_INVALID_ARG;
    ctx->bvh_leaf = leaf_max;
    if (!ctx->have_scene) return PPM_OK;
    cudaSetDevice(ctx->device);
    ctx->render_ready = false;
    drop_graph(ctx);
    return build_accel(ctx);
}

// Leaf-size autotuner: rebuilds the tree with 1, 2, 4 and 8 objects per leaf,
// times the FP32 first-hit kernel over the caller's rays (best of two) and
// keeps the fastest tree.
extern "C" int ppm_tune_bvh_leaf(ppm_ctx *ctx, const double *rays, int64_t n, int32_t *best_leaf, double *best_ms) {
    if (!ctx || !rays || n <= 0) return PPM_ERR_INVALID_ARG;
    if (!ctx->have_scene) return set_err(ctx, PPM_ERR_NOT_READY, "no scene");
    cudaSetDevice(ctx->device);
    const size_t rb = sizeof(double) * 6 * n, tb = sizeof(double) * n, ob = sizeof(int32_t) * n;
    TRY(ensure(ctx, ctx->scratch, rb + tb + ob + 64));
    char *base = as<char>(ctx->scratch);
    double *d_r = (double *)base, *d_t = (double *)(base + rb);
    int32_t *d_o = (int32_t *)(base + rb + tb);
    CK(cudaMemcpyAsync(d_r, rays, rb, cudaMemcpyHostToDevice, ctx->s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return set_err(ctx, PPM_ERR_CUDA, "event"); }
    int best = ctx->bvh_leaf, rc = PPM_OK;
    float best_t = 1e30f;
    for (int leaf : {1, 2, 4, 8}) {
        ctx->bvh_leaf = leaf;
        if ((rc = build_accel(ctx)) != PPM_OK) break;
        float t = 1e30f;
        for (int rep = 0; rep < 2 && rc == PPM_OK; rep++) {
            float ms = 0.0f;
            cudaError_t e = cudaEventRecord(e0, ctx->s);
            if (e == cudaSuccess) launch_intersect_f(ctx->sv_f, d_r, n, d_t, d_o, ctx->s);
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) rc = set_err(ctx, PPM_ERR_CUDA, "leaf tuner: %s", cudaGetErrorString(e));
            t = std::min(t, ms);
        }
        if (rc == PPM_OK && t < best_t) { best_t = t; best = leaf; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != PPM_OK) return rc;
    ctx->bvh_leaf = best;
    ctx->render_ready = false;
    drop_graph(ctx);
    TRY(build_accel(ctx));
    if (best_leaf) *best_leaf = best;
    if (best_ms) *best_ms = best_t;
    return PPM_OK;
}

extern "C" int ppm_accel_info(ppm_ctx *ctx, int32_t *bvh_objects, int32_t *unbounded) {
    if (!ctx) return PPM_ERR_INVALID_ARG;
    if (bvh_objects) *bvh_objects = ctx->bvh_m;
    if (unbounded) *unbounded = ctx->sv_d.n_unb;
    return PPM_OK;
}

extern "C" int ppm_camera_set(ppm_ctx *ctx, const ppm_camera *cam) {
    if (!ctx || !cam) return PPM_ERR_INVALID_ARG;
    if (cam->xreso <= 0 || cam->yreso <= 0 || (long long)cam->xreso * cam->yreso > (1LL << 28))
        return set_err(ctx, PPM_ERR_INVALID_ARG, "bad resolution %dx%d", cam->xreso, cam->yreso);
    ctx->cam = *cam;
    ppm_camera_derive(&ctx->cam);
    conv_camera(ctx->cam, ctx->cam_d);
    conv_camera(ctx->cam, ctx->cam_f);
    ctx->have_cam = true;
    ctx->render_ready = false;
    drop_graph(ctx);
    return PPM_OK;
}

// ---------------------------------------------------------------------------
// FP64 parity entry points
// ---------------------------------------------------------------------------
extern "C" int ppm_intersect(ppm_ctx *ctx, const double *rays, int64_t n, double *t, int32_t *obj, double *nrm) {
    if (!ctx || n < 0 || (n && (!rays || !t || !obj))) return PPM_ERR_INVALID_ARG;
    if (!ctx->have_scene) return set_err(ctx, PPM_ERR_NOT_READY, "no scene uploaded");
    if (n == 0) return PPM_OK;
    cudaSetDevice(ctx->device);
    size_t rb = sizeof(double) * 6 * n, tb = sizeof(double) * n, ob = sizeof(int32_t) * n, nb = sizeof(double) * 3 * n;
    TRY(ensure(ctx, ctx->scratch, rb + tb + ob + nb + 64));
    char *base = as<char>(ctx->scratch);
    double *d_rays = (double *)base, *d_t = (double *)(base + rb);
    double *d_n = (double *)(base + rb + tb);
    int32_t *d_o = (int32_t *)(base + rb + tb + nb);
    CK(cudaMemcpyAsync(d_rays, rays, rb, cudaMemcpyHostToDevice, ctx->s));
    launch_intersect_d(ctx->sv_d, d_rays, n, d_t, d_o, nrm ? d_n : nullptr, ctx->s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(t, d_t, tb, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(obj, d_o, ob, cudaMemcpyDeviceToHost, ctx->s));
    if (nrm) CK(cudaMemcpyAsync(nrm, d_n, nb, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PPM_OK;
}

extern "C" int ppm_intersect_f32(ppm_ctx *ctx, const double *rays, int64_t n, double *t, int32_t *obj) {
    if (!ctx || n < 0 || (n && (!rays || !t || !obj))) return PPM_ERR_INVALID_ARG;
    if (!ctx->have_scene) return set_err(ctx, PPM_ERR_NOT_READY, "no scene uploaded");
    if (n == 0) return PPM_OK;
    cudaSetDevice(ctx->device);
    size_t rb = sizeof(double) * 6 * n, tb = sizeof(double) * n, ob = sizeof(int32_t) * n;
    TRY(ensure(ctx, ctx->scratch, rb + tb + ob + 64));
    char *base = as<char>(ctx->scratch);
    double *d_rays = (double *)base, *d_t = (double *)(base + rb);
    int32_t *d_o = (int32_t *)(base + rb + tb);
    CK(cudaMemcpyAsync(d_rays, rays, rb, cudaMemcpyHostToDevice, ctx->s));
    launch_intersect_f(ctx->sv_f, d_rays, n, d_t, d_o, ctx->s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(t, d_t, tb, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(obj, d_o, ob, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PPM_OK;
}

static int ensure_photons_d(ppm_ctx *ctx, long long cap) {
    TRY(ensure(ctx, ctx->raw_d, sizeof(PhotonD) * cap));
    TRY(ensure(ctx, ctx->spos, sizeof(double4) * cap));
    TRY(ensure(ctx, ctx->sdir, sizeof(double4) * cap));
    TRY(ensure(ctx, ctx->keyrank, sizeof(uint2) * cap));
    ctx->photon_cap_d = std::max(ctx->photon_cap_d, cap);
    return ensure_grid(ctx);
}

static int ensure_photons_f(ppm_ctx *ctx, long long cap, bool with_idx) {
    TRY(ensure(ctx, ctx->raw_f, sizeof(float4) * cap));
    TRY(ensure(ctx, ctx->sorted_f, sizeof(float4) * cap));
    TRY(ensure(ctx, ctx->keyrank, sizeof(uint2) * cap));
    if (with_idx) TRY(ensure(ctx, ctx->sidx, sizeof(int32_t) * cap));
    ctx->photon_cap_f = std::max(ctx->photon_cap_f, cap);
    return ensure_grid(ctx);
}

extern "C" int ppm_trace_photons(ppm_ctx *ctx, int64_t nphoton, int32_t use_classic, uint32_t pass, int64_t *n_stored,
                                 double *power, int64_t *n_emitted) {
    if (!ctx || nphoton <= 0) return PPM_ERR_INVALID_ARG;
    if (!ctx->have_scene || ctx->lights.empty()) return set_err(ctx, PPM_ERR_NOT_READY, "no scene with lights");
    cudaSetDevice(ctx->device);
    EmitPlan plan;
    double pw = make_plan(ctx->lights, nphoton, plan);
    long long nem = plan.first[plan.n_lights];
    if (nem > 0x7fffffffLL) return set_err(ctx, PPM_ERR_INVALID_ARG, "too many photons");
    long long cap = std::max(1LL, nem * MAX_TRACE);
    TRY(ensure_photons_d(ctx, cap));
    TRY(upload_state(ctx, 0.0, (int)pass, 0.0, 1, 1.0, cap, 0));
    launch_pass_begin(ctx->st, ctx->s);
    PhotonBuf<double> pb{as<PhotonD>(ctx->raw_d), as<double4>(ctx->spos), as<double4>(ctx->sdir)};
    enqueue_photon_trace<double>(ctx, plan, ctx->seed, use_classic ? 1 : 0, pb, ctx->s);
    CK(cudaGetLastError());
    PassState h;
    TRY(read_state(ctx, h));
    if (h.overflow & 1u) return set_err(ctx, PPM_ERR_CAPACITY, "photon buffer overflow");
    ctx->map_n = (long long)h.n_stored;
    ctx->last_trace_pw = pw;
    ctx->last_trace_uc = use_classic;
    if (n_stored) *n_stored = (int64_t)h.n_stored;
    if (power) *power = pw;
    if (n_emitted) *n_emitted = nem;
    ctx->map_kind = 0;
    return PPM_OK;
}

extern "C" int ppm_photons_download(ppm_ctx *ctx, double *pos, double *dir, uint8_t *wl, int32_t *emit_idx,
                                    int8_t *level, int64_t cap) {
    if (!ctx) return PPM_ERR_INVALID_ARG;
    long long n = ctx->map_n;
    if (cap < n) return set_err(ctx, PPM_ERR_CAPACITY, "need room for %lld photons", n);
    std::vector<PhotonD> h((size_t)n);
    if (n) {
        CK(cudaMemcpyAsync(h.data(), ctx->raw_d.p, sizeof(PhotonD) * n, cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    for (long long i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) {
            if (pos) pos[3 * i + a] = h[i].pos[a];
            if (dir) dir[3 * i + a] = h[i].dir[a];
        }
        if (wl) wl[i] = h[i].wl;
        if (emit_idx) emit_idx[i] = h[i].emit;
        if (level) level[i] = h[i].level;
    }
    return PPM_OK;
}

// build the sorted FP64 map from raw_d[0, n)
static int build_map_d(ppm_ctx *ctx, long long n, double r2, double pw) {
    PhotonBuf<double> pb{as<PhotonD>(ctx->raw_d), as<double4>(ctx->spos), as<double4>(ctx->sdir)};
    TRY(upload_state(ctx, r2, 0, 0.0, 1, 1.0, n, 0));
    launch_pass_begin(ctx->st, ctx->s);
    int g = grid_blocks(ctx, 4);
    launch_bbox_d(pb, ctx->st, n, g, ctx->s);
    launch_grid_setup(ctx->st, r2, ctx->s);
    launch_hist_d(pb, ctx->st, n, as<uint32_t>(ctx->count), as<uint2>(ctx->keyrank), g, ctx->s);
    launch_scan(as<uint32_t>(ctx->count), ctx->st, as<uint32_t>(ctx->block_sums), as<uint32_t>(ctx->start), CELL_CAP,
                ctx->s, grid_blocks(ctx, 8));
    launch_scatter_d(pb, ctx->st, n, as<uint32_t>(ctx->start), as<uint2>(ctx->keyrank), g, ctx->s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->s));
    ctx->map_kind = 1;
    ctx->map_n = n;
    ctx->map_pw = pw;
    ctx->map_r2 = r2;
    return PPM_OK;
}

extern "C" int ppm_photonmap_build(ppm_ctx *ctx, const double *pos, const double *dir, const uint8_t *wl, int64_t n,
                                   double power, double radius2) {
    if (!ctx || n < 0 || (n && (!pos || !dir || !wl)) || !(radius2 > 0.0)) return PPM_ERR_INVALID_ARG;
    if (n > 0x7fffffffLL) return set_err(ctx, PPM_ERR_INVALID_ARG, "at most 2^31-1 photons");
    cudaSetDevice(ctx->device);
    drop_graph(ctx);
    ctx->render_ready = false;
    TRY(ensure_photons_d(ctx, std::max<long long>(n, 1)));
    std::vector<PhotonD> h((size_t)n);
    for (long long i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) { h[i].pos[a] = pos[3 * i + a]; h[i].dir[a] = dir[3 * i + a]; }
        if (wl[i] > 2) return set_err(ctx, PPM_ERR_INVALID_ARG, "photon %lld: wavelength %d > 2", i, (int)wl[i]);
        h[i].wl = wl[i];
        h[i].emit = (int32_t)i;
        h[i].level = 0;
        h[i].pad = 0;
    }
    if (n) CK(cudaMemcpyAsync(ctx->raw_d.p, h.data(), sizeof(PhotonD) * n, cudaMemcpyHostToDevice, ctx->s));
    return build_map_d(ctx, n, radius2, power);
}

extern "C" int ppm_photonmap_from_trace(ppm_ctx *ctx, double radius2) {
    if (!ctx || !(radius2 > 0.0)) return PPM_ERR_INVALID_ARG;
    if (ctx->raw_d.p == nullptr) return set_err(ctx, PPM_ERR_NOT_READY, "no traced photons");
    cudaSetDevice(ctx->device);
    return build_map_d(ctx, ctx->map_n, radius2, ctx->last_trace_pw);
}

static int check_r2(ppm_ctx *ctx, const double *r2, int64_t nq) {
    for (int64_t i = 0; i < nq; i++)
        if (!(r2[i] >= 0.0) || r2[i] > ctx->map_r2 * (1.0 + 1e-12))
            return set_err(ctx, PPM_ERR_INVALID_ARG, "query %lld: r2 %.17g outside [0, map radius2 %.17g]", (long long)i,
                           r2[i], ctx->map_r2);
    return PPM_OK;
}

// shared count -> offsets -> fill flow for both map precisions
template <typename Launch>
static int within_flow(ppm_ctx *ctx, int64_t nq, int64_t *offsets, int32_t *idx, int64_t cap, int64_t *total,
                       char *d_base, Launch launch) {
    unsigned long long *d_counts = (unsigned long long *)d_base;
    launch(d_counts, (const unsigned long long *)nullptr, (int32_t *)nullptr);
    CK(cudaGetLastError());
    std::vector<unsigned long long> cnt((size_t)nq);
    if (nq) CK(cudaMemcpyAsync(cnt.data(), d_counts, sizeof(unsigned long long) * nq, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    std::vector<unsigned long long> off((size_t)nq + 1);
    unsigned long long run = 0;
    for (int64_t i = 0; i < nq; i++) { off[i] = run; run += cnt[i]; }
    off[nq] = run;
    if (total) *total = (int64_t)run;
    if (offsets)
        for (int64_t i = 0; i <= nq; i++) offsets[i] = (int64_t)off[i];
    if (!idx) return PPM_OK;
    if ((int64_t)run > cap) return set_err(ctx, PPM_ERR_CAPACITY, "idx needs %llu entries, cap %lld", run, (long long)cap);
    DevBuf out;
    // index section rounded up to 16 bytes so the u64 offsets after it stay aligned
    size_t ob = (sizeof(int32_t) * (run ? run : 1) + 15) & ~(size_t)15, fb = sizeof(unsigned long long) * (nq + 1);
    if (cudaMalloc(&out.p, ob + fb) != cudaSuccess) return set_err(ctx, PPM_ERR_OOM, "no memory for %llu indices", run);
    int32_t *d_idx = (int32_t *)out.p;
    unsigned long long *d_off = (unsigned long long *)((char *)out.p + ob);
    cudaMemcpyAsync(d_off, off.data(), fb, cudaMemcpyHostToDevice, ctx->s);
    launch((unsigned long long *)nullptr, (const unsigned long long *)d_off, d_idx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx, d_idx, sizeof(int32_t) * run, cudaMemcpyDeviceToHost, ctx->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->s);
    cudaFree(out.p);
    if (e != cudaSuccess) return set_err(ctx, PPM_ERR_CUDA, "within fill: %s", cudaGetErrorString(e));
    for (int64_t i = 0; i < nq; i++) std::sort(idx + off[i], idx + off[i + 1]);
    return PPM_OK;
}

extern "C" int ppm_query_within(ppm_ctx *ctx, const double *q, int64_t nq, const double *r2, int64_t *offsets,
                                int32_t *idx, int64_t cap, int64_t *total) {
    if (!ctx || nq < 0 || (nq && (!q || !r2))) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 1) return set_err(ctx, PPM_ERR_NOT_READY, "no FP64 photon map built");
    TRY(check_r2(ctx, r2, nq));
    cudaSetDevice(ctx->device);
    size_t qb = sizeof(double) * 3 * nq, rb = sizeof(double) * nq, cb = sizeof(unsigned long long) * (nq + 1);
    TRY(ensure(ctx, ctx->scratch, qb + rb + cb + 64));
    char *base = as<char>(ctx->scratch);
    double *d_q = (double *)base, *d_r2 = (double *)(base + qb);
    if (nq) {
        CK(cudaMemcpyAsync(d_q, q, qb, cudaMemcpyHostToDevice, ctx->s));
        CK(cudaMemcpyAsync(d_r2, r2, rb, cudaMemcpyHostToDevice, ctx->s));
    }
    int g = grid_blocks(ctx, 8);
    return within_flow(ctx, nq, offsets, idx, cap, total, base + qb + rb,
                       [&](unsigned long long *counts, const unsigned long long *off, int32_t *out) {
                           launch_within_d(d_q, nq, d_r2, ctx->st, as<double4>(ctx->spos), as<uint32_t>(ctx->start),
                                           counts, off, out, g, ctx->s);
                       });
}

extern "C" int ppm_estimate(ppm_ctx *ctx, const double *pos, const double *nrm, int64_t nq, int32_t pfilter,
                            double *rgb) {
    if (!ctx || nq < 0 || (nq && (!pos || !nrm || !rgb)) || pfilter < 0 || pfilter > 2) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 1) return set_err(ctx, PPM_ERR_NOT_READY, "no FP64 photon map built");
    if (nq == 0) return PPM_OK;
    cudaSetDevice(ctx->device);
    size_t pb = sizeof(double) * 3 * nq, hb = sizeof(HitPoint<double>) * nq, ob = sizeof(double) * 3 * nq;
    TRY(ensure(ctx, ctx->scratch, 2 * pb + hb + ob + 256));
    char *base = as<char>(ctx->scratch);
    double *d_p = (double *)base, *d_n = (double *)(base + pb);
    HitPoint<double> *d_h = (HitPoint<double> *)(base + 2 * pb);
    double *d_o = (double *)(base + 2 * pb + hb);
    CK(cudaMemcpyAsync(d_p, pos, pb, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(d_n, nrm, pb, cudaMemcpyHostToDevice, ctx->s));
    launch_make_queries_d(d_p, d_n, nq, d_h, ctx->s);
    GatherOutD go{nullptr, d_o, nullptr};
    launch_gather_d(d_h, ctx->st, nq, as<double4>(ctx->spos), as<double4>(ctx->sdir), as<uint32_t>(ctx->start),
                    ctx->map_pw, pfilter, 1, go, grid_blocks(ctx, 8), ctx->s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rgb, d_o, ob, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PPM_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free estimate.
//
// ppm_estimate stages its queries and results in the context's scratch
// buffer, which it frees and re-allocates whenever a call is larger than any
// before it.  Some callers cannot have the library allocate at that point:
// a host that has already given nearly all device memory to its own pool
// (where a cudaMalloc could fail in the middle of a run), or one running
// other streams on the same GPU that cannot take the device-wide wait a
// cudaFree implies.  ppm_estimate_noalloc computes the same estimates from a
// fixed array in device memory instead, so it never allocates or frees.
//
// The array is one per device, shared by every context and every call in
// this process.  ppm_ctx_create looks up its device address (with the
// context's device current) and keeps it in the context: the lookup is what
// loads this file's module onto the device and places the array there, so
// that happens when the context is created, not in the middle of a run.  A
// context created after a cudaDeviceReset looks the address up again.
// Calls whose GPU work overlaps -- from two host threads, or two contexts on
// the same device -- race on the array and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace {

// Per-query staging: position and normal as the caller passes them, the hit
// point the gather reads, and the output row.  Each section is sized for the
// maximum query count, so every section starts on a 256-byte boundary.
constexpr size_t NOALLOC_Q = PPM_ESTIMATE_NOALLOC_MAX_QUERIES;
constexpr size_t NOALLOC_POS_OFF = 0;
constexpr size_t NOALLOC_NRM_OFF = NOALLOC_POS_OFF + sizeof(double) * 3 * NOALLOC_Q;
constexpr size_t NOALLOC_HIT_OFF = NOALLOC_NRM_OFF + sizeof(double) * 3 * NOALLOC_Q;
constexpr size_t NOALLOC_OUT_OFF = NOALLOC_HIT_OFF + sizeof(HitPoint<double>) * NOALLOC_Q;
constexpr size_t NOALLOC_BYTES = NOALLOC_OUT_OFF + sizeof(double) * 3 * NOALLOC_Q;
static_assert(NOALLOC_NRM_OFF % 256 == 0 && NOALLOC_HIT_OFF % 256 == 0 && NOALLOC_OUT_OFF % 256 == 0,
              "staging sections must stay 256-byte aligned");

}  // namespace

static __device__ __align__(256) unsigned char g_estimate_scratch[NOALLOC_BYTES];

// Device address of g_estimate_scratch on the current device (called by
// ppm_ctx_create with the context's device current).
static cudaError_t noalloc_lookup(char **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_estimate_scratch);
    if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
    *out = e == cudaSuccess ? static_cast<char *>(p) : nullptr;
    return e;
}

extern "C" int ppm_estimate_noalloc(ppm_ctx *ctx, const double *pos, const double *nrm, int64_t nq,
                                    int32_t pfilter, double *rgb) {
    if (!ctx || nq < 0 || (nq && (!pos || !nrm || !rgb)) || pfilter < 0 || pfilter > 2) return PPM_ERR_INVALID_ARG;
    if (nq > PPM_ESTIMATE_NOALLOC_MAX_QUERIES)
        return set_err(ctx, PPM_ERR_INVALID_ARG,
                       "%lld queries: the allocation-free estimate takes at most %d per call (split the batch "
                       "or use ppm_estimate)", (long long)nq, PPM_ESTIMATE_NOALLOC_MAX_QUERIES);
    if (ctx->map_kind != 1) return set_err(ctx, PPM_ERR_NOT_READY, "no FP64 photon map built");
    if (nq == 0) return PPM_OK;
    CK(cudaSetDevice(ctx->device));
    char *base = ctx->noalloc_base;   // looked up by ppm_ctx_create
    if (!base) return set_err(ctx, PPM_ERR_NOT_READY, "the allocation-free estimate's array is not placed on device %d",
                              ctx->device);
    double *d_p = (double *)(base + NOALLOC_POS_OFF), *d_n = (double *)(base + NOALLOC_NRM_OFF);
    HitPoint<double> *d_h = (HitPoint<double> *)(base + NOALLOC_HIT_OFF);
    double *d_o = (double *)(base + NOALLOC_OUT_OFF);
    size_t pb = sizeof(double) * 3 * nq;
    CK(cudaMemcpyAsync(d_p, pos, pb, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(d_n, nrm, pb, cudaMemcpyHostToDevice, ctx->s));
    // The gather writes every output row it owns; the rows are cleared anyway
    // so that no row can ever carry an earlier call's value.
    CK(cudaMemsetAsync(d_o, 0, pb, ctx->s));
    launch_make_queries_d(d_p, d_n, nq, d_h, ctx->s);
    GatherOutD go{nullptr, d_o, nullptr};
    launch_gather_d(d_h, ctx->st, nq, as<double4>(ctx->spos), as<double4>(ctx->sdir), as<uint32_t>(ctx->start),
                    ctx->map_pw, pfilter, 1, go, grid_blocks(ctx, 8), ctx->s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rgb, d_o, pb, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PPM_OK;
}

// One eye pass over the FP64 photon map of ppm_photonmap_build: what the
// reference's `rt` does with a map read from `pm` (src/bin/rt.rs:41-46):
// trace_ray (tracer.rs:129-177) for every pixel's camera ray, with the map's
// power and radius^2 in the estimate.  pass selects the random streams.
extern "C" int ppm_eye_pass(ppm_ctx *ctx, int32_t use_classic, uint64_t seed, int32_t pass, double *image_out) {
    if (!ctx || !image_out || pass < 0) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 1) return set_err(ctx, PPM_ERR_NOT_READY, "no FP64 photon map built");
    if (!ctx->have_scene || !ctx->have_cam) return set_err(ctx, PPM_ERR_NOT_READY, "scene and camera must be set");
    cudaSetDevice(ctx->device);
    drop_graph(ctx);
    ctx->render_ready = false;
    ctx->npx = (long long)ctx->cam.xreso * ctx->cam.yreso;
    ctx->hit_cap = ctx->npx * HITS_PER_PIXEL;
    TRY(ensure(ctx, ctx->hits_d, sizeof(HitPoint<double>) * ctx->hit_cap));
    TRY(ensure_eye_queues(ctx, ctx->npx, sizeof(double4)));
    TRY(ensure(ctx, ctx->pass_img, sizeof(double) * 3 * ctx->npx));
    // the map's grid and radius stay; the eye needs the hit capacity and pass
    const unsigned long long hcap = (unsigned long long)ctx->hit_cap;
    CK(cudaMemcpyAsync(&ctx->st->hit_cap, &hcap, sizeof hcap, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(&ctx->st->pass, &pass, sizeof pass, cudaMemcpyHostToDevice, ctx->s));
    launch_pass_begin(ctx->st, ctx->s);
    const int uc = use_classic ? 1 : 0;
    enqueue_eye<double>(ctx, as<HitPoint<double>>(ctx->hits_d),
        [&](int l, EyeQueue<double> in, EyeQueue<double> out, unsigned long long qcap, HitPoint<double> *h, int g,
            cudaStream_t st) {
            launch_eye_level_d(ctx->sv_d, ctx->cam_d, seed, ctx->st, uc, l, in, out, qcap, h,
                               EyeOut<double>{as<double>(ctx->pass_img)}, g, st);
        }, ctx->s);
    GatherOutD go{as<double>(ctx->pass_img), nullptr, nullptr};
    launch_gather_d(as<HitPoint<double>>(ctx->hits_d), ctx->st, -1, as<double4>(ctx->spos), as<double4>(ctx->sdir),
                    as<uint32_t>(ctx->start), ctx->map_pw, ctx->cam.pfilter, 0, go, grid_blocks(ctx, 8), ctx->s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(image_out, ctx->pass_img.p, sizeof(double) * 3 * ctx->npx, cudaMemcpyDeviceToHost, ctx->s));
    PassState h;
    TRY(read_state(ctx, h));
    if (h.overflow) return set_err(ctx, PPM_ERR_CAPACITY, "eye pass overflow (flags %u)", h.overflow);
    return PPM_OK;
}

// ---------------------------------------------------------------------------
// FP32 photon map (gather sweep)
// ---------------------------------------------------------------------------
// Sorts the packed photons in raw_f into cells of r_max / k (bounds, cell
// histogram, scan, scatter); the map's original order stays in raw_f, so the
// grid can be rebuilt with another k without the host arrays.
static int grid_map_f32(ppm_ctx *ctx, long long n, double r2max, double k) {
    PhotonBuf<float> pb{as<float4>(ctx->raw_f), as<float4>(ctx->sorted_f), as<int32_t>(ctx->sidx)};
    TRY(upload_state(ctx, r2max, 0, 0.0, 1, k, n, 0, 1, CELL_CAP / 3));
    launch_pass_begin(ctx->st, ctx->s);
    int g = grid_blocks(ctx, 4);
    launch_bbox_f(pb, ctx->st, n, g, ctx->s);
    launch_grid_setup(ctx->st, r2max, ctx->s);
    launch_hist_f(pb, ctx->st, n, as<uint32_t>(ctx->count), as<uint2>(ctx->keyrank), g, ctx->s);
    launch_scan(as<uint32_t>(ctx->count), ctx->st, as<uint32_t>(ctx->block_sums), as<uint32_t>(ctx->start), CELL_CAP,
                ctx->s, grid_blocks(ctx, 8));
    launch_scatter_f(pb, ctx->st, n, as<uint32_t>(ctx->start), as<uint2>(ctx->keyrank), g, ctx->s);
    CK(cudaGetLastError());
    return PPM_OK;
}

extern "C" int ppm_photonmap_build_f32(ppm_ctx *ctx, const float *pos, const float *dir, const uint8_t *wl, int64_t n,
                                       double power, double radius2_max) {
    if (!ctx || n < 0 || (n && (!pos || !dir || !wl)) || !(radius2_max > 0.0)) return PPM_ERR_INVALID_ARG;
    if (n > 0x7fffffffLL) return set_err(ctx, PPM_ERR_INVALID_ARG, "at most 2^31-1 photons");
    for (int64_t i = 0; i < n; i++)
        if (wl[i] > 2) return set_err(ctx, PPM_ERR_INVALID_ARG, "photon %lld: wavelength %d > 2", (long long)i, (int)wl[i]);
    cudaSetDevice(ctx->device);
    drop_graph(ctx);
    ctx->render_ready = false;
    TRY(ensure_photons_f(ctx, std::max<long long>(n, 1), true));
    // stage host arrays (pos, dir: 12 B each, wl: 1 B) and pack on the device
    size_t vb = sizeof(float) * 3 * n;
    TRY(ensure(ctx, ctx->scratch, 2 * vb + n + 64));
    char *base = as<char>(ctx->scratch);
    float *d_pos = (float *)base, *d_dir = (float *)(base + vb);
    uint8_t *d_wl = (uint8_t *)(base + 2 * vb);
    if (n) {
        CK(cudaMemcpyAsync(d_pos, pos, vb, cudaMemcpyHostToDevice, ctx->s));
        CK(cudaMemcpyAsync(d_dir, dir, vb, cudaMemcpyHostToDevice, ctx->s));
        CK(cudaMemcpyAsync(d_wl, wl, n, cudaMemcpyHostToDevice, ctx->s));
    }
    launch_pack_photons_f(d_pos, d_dir, d_wl, n, as<float4>(ctx->raw_f), ctx->s);
    if (ctx->timing) CK(cudaEventRecord(ctx->xev[0], ctx->s));
    TRY(grid_map_f32(ctx, n, radius2_max, ctx->map_cells));
    if (ctx->timing) CK(cudaEventRecord(ctx->xev[1], ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (ctx->timing) TRY(add_stage_time(ctx, 1, ctx->xev[0], ctx->xev[1]));
    ctx->map_kind = 2;
    ctx->map_n = n;
    ctx->map_pw = power;
    ctx->map_r2 = radius2_max;
    return PPM_OK;
}

extern "C" int ppm_photonmap_regrid_f32(ppm_ctx *ctx, double cells_per_radius) {
    if (!ctx || !(cells_per_radius >= 0.5 && cells_per_radius <= 8.0)) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 2) return set_err(ctx, PPM_ERR_NOT_READY, "no FP32 photon map built");
    cudaSetDevice(ctx->device);
    TRY(grid_map_f32(ctx, ctx->map_n, ctx->map_r2, cells_per_radius));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->map_cells = cells_per_radius;
    return PPM_OK;
}

extern "C" int ppm_query_within_f32(ppm_ctx *ctx, const float *q, int64_t nq, const double *r2, int64_t *offsets,
                                    int32_t *idx, int64_t cap, int64_t *total) {
    if (!ctx || nq < 0 || (nq && (!q || !r2))) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 2) return set_err(ctx, PPM_ERR_NOT_READY, "no FP32 photon map built");
    TRY(check_r2(ctx, r2, nq));
    cudaSetDevice(ctx->device);
    size_t qb = sizeof(float) * 3 * nq, rb = sizeof(double) * nq, cb = sizeof(unsigned long long) * (nq + 1);
    qb = (qb + 15) & ~(size_t)15;
    TRY(ensure(ctx, ctx->scratch, qb + rb + cb + 64));
    char *base = as<char>(ctx->scratch);
    float *d_q = (float *)base;
    double *d_r2 = (double *)(base + qb);
    if (nq) {
        CK(cudaMemcpyAsync(d_q, q, sizeof(float) * 3 * nq, cudaMemcpyHostToDevice, ctx->s));
        CK(cudaMemcpyAsync(d_r2, r2, rb, cudaMemcpyHostToDevice, ctx->s));
    }
    int g = grid_blocks(ctx, 8);
    return within_flow(ctx, nq, offsets, idx, cap, total, base + qb + rb,
                       [&](unsigned long long *counts, const unsigned long long *off, int32_t *out) {
                           launch_within_f(d_q, nq, d_r2, ctx->st, as<float4>(ctx->sorted_f), as<uint32_t>(ctx->start),
                                           as<int32_t>(ctx->sidx), counts, off, out, g, ctx->s);
                       });
}

// Device staging of an FP32 estimate batch in the scratch buffer.
struct EstBatch {
    float *p, *n;
    double *r2, *r2s, *o;
    HitPoint<float> *h;
    uint2 *kr;
};

static int stage_estimate_f32(ppm_ctx *ctx, const float *pos, const float *nrm, int64_t nq, const double *r2,
                              EstBatch &b) {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t pb = al(sizeof(float) * 3 * nq), hb = al(sizeof(HitPoint<float>) * nq);
    const size_t rb = al(sizeof(double) * nq), kb = al(sizeof(uint2) * nq), ob = sizeof(double) * 3 * nq;
    TRY(ensure(ctx, ctx->scratch, 2 * pb + hb + 2 * rb + kb + ob + 256));
    TRY(ensure(ctx, ctx->qstart, sizeof(uint32_t) * (CELL_CAP + 1)));
    char *base = as<char>(ctx->scratch);
    b.p = (float *)base;
    b.n = (float *)(base + pb);
    b.h = (HitPoint<float> *)(base + 2 * pb);
    b.r2 = (double *)(base + 2 * pb + hb);
    b.r2s = (double *)(base + 2 * pb + hb + rb);
    b.kr = (uint2 *)(base + 2 * pb + hb + 2 * rb);
    b.o = (double *)(base + 2 * pb + hb + 2 * rb + kb);
    CK(cudaMemcpyAsync(b.p, pos, sizeof(float) * 3 * nq, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(b.n, nrm, sizeof(float) * 3 * nq, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(b.r2, r2, sizeof(double) * nq, cudaMemcpyHostToDevice, ctx->s));
    return PPM_OK;
}

// Queries are sorted by map cell on the device before the gather (see
// k_query_hist), so results land in the caller's order whatever the order of
// the gather.  e0/e1/e2 (optional) bracket the sort and the gather.
static int run_estimate_f32(ppm_ctx *ctx, const EstBatch &b, int64_t nq, bool count, cudaEvent_t e0, cudaEvent_t e1,
                            cudaEvent_t e2) {
    if (e0) CK(cudaEventRecord(e0, ctx->s));
    launch_query_sort_f(b.p, b.n, b.r2, nq, ctx->st, ctx->map_r2, as<uint32_t>(ctx->count),
                        as<uint32_t>(ctx->block_sums), as<uint32_t>(ctx->qstart), CELL_CAP, b.kr, b.h, b.r2s,
                        grid_blocks(ctx, 8), ctx->s);
    GatherOutF go{nullptr, b.o, nullptr};
    if (count) {
        CK(cudaMemsetAsync(&ctx->st->candidates, 0, 3 * sizeof(unsigned long long), ctx->s));
        go.count = &ctx->st->candidates;
    }
    CK(cudaMemsetAsync(&ctx->st->gather_next, 0, sizeof(unsigned long long), ctx->s));
    if (e1) CK(cudaEventRecord(e1, ctx->s));
    launch_estimate_tile_f(b.h, b.r2s, nq, ctx->st, as<float4>(ctx->sorted_f), as<uint32_t>(ctx->start), ctx->map_pw,
                           go, grid_blocks(ctx, ctx->est_blocks), ctx->s);
    CK(cudaGetLastError());
    if (e2) CK(cudaEventRecord(e2, ctx->s));
    return PPM_OK;
}

extern "C" int ppm_estimate_f32(ppm_ctx *ctx, const float *pos, const float *nrm, int64_t nq, const double *r2,
                                double *rgb) {
    if (!ctx || nq < 0 || (nq && (!pos || !nrm || !r2 || !rgb))) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 2) return set_err(ctx, PPM_ERR_NOT_READY, "no FP32 photon map built");
    if (nq > 0x7fffffffLL) return set_err(ctx, PPM_ERR_INVALID_ARG, "at most 2^31-1 queries per call");
    TRY(check_r2(ctx, r2, nq));
    if (nq == 0) return PPM_OK;
    cudaSetDevice(ctx->device);
    EstBatch b;
    TRY(stage_estimate_f32(ctx, pos, nrm, nq, r2, b));
    const bool t = ctx->timing;
    TRY(run_estimate_f32(ctx, b, nq, ctx->count_gather, t ? ctx->xev[0] : nullptr, t ? ctx->xev[1] : nullptr,
                         t ? ctx->xev[2] : nullptr));
    CK(cudaMemcpyAsync(rgb, b.o, sizeof(double) * 3 * nq, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (t) {
        TRY(add_stage_time(ctx, 5, ctx->xev[0], ctx->xev[1]));
        TRY(add_stage_time(ctx, 3, ctx->xev[1], ctx->xev[2]));
    }
    return PPM_OK;
}

// Gather cell-size autotuner: re-grids the map with each candidate number of
// cells per maximum radius, times sort + gather of the sample on the device
// (best of three), and keeps the fastest grid.  Smaller cells cut the
// candidates a query tests; larger cells cut rows and scan overhead and fit
// clustered maps whose dense cells would otherwise hit the cell cap.
extern "C" int ppm_photonmap_tune_f32(ppm_ctx *ctx, const float *pos, const float *nrm, int64_t nq, const double *r2,
                                      double *best_cells, double *best_ms) {
    if (!ctx || nq <= 0 || !pos || !nrm || !r2) return PPM_ERR_INVALID_ARG;
    if (ctx->map_kind != 2) return set_err(ctx, PPM_ERR_NOT_READY, "no FP32 photon map built");
    if (nq > 0x7fffffffLL) return set_err(ctx, PPM_ERR_INVALID_ARG, "at most 2^31-1 queries");
    TRY(check_r2(ctx, r2, nq));
    cudaSetDevice(ctx->device);
    cudaEvent_t e[2];
    CK(cudaEventCreate(&e[0]));
    if (cudaEventCreate(&e[1]) != cudaSuccess) {
        cudaEventDestroy(e[0]);
        return set_err(ctx, PPM_ERR_CUDA, "cudaEventCreate failed");
    }
    const double cand[] = {1.0, 1.5, 2.0, 3.0, 4.0};
    double best = ctx->map_cells, best_t = 1e30;
    int rc = PPM_OK;
    EstBatch b;
    rc = stage_estimate_f32(ctx, pos, nrm, nq, r2, b);
    for (double k : cand) {
        if (rc != PPM_OK) break;
        if ((rc = grid_map_f32(ctx, ctx->map_n, ctx->map_r2, k)) != PPM_OK) break;
        float t = 1e30f;
        for (int rep = 0; rep < 3 && rc == PPM_OK; rep++) {
            if ((rc = run_estimate_f32(ctx, b, nq, false, e[0], nullptr, e[1])) != PPM_OK) break;
            float ms = 0.0f;
            cudaError_t ce = cudaEventSynchronize(e[1]);
            if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e[0], e[1]);
            if (ce != cudaSuccess) rc = set_err(ctx, PPM_ERR_CUDA, "tuner timing: %s", cudaGetErrorString(ce));
            t = std::min(t, ms);
        }
        if (rc == PPM_OK && t < best_t) { best_t = t; best = k; }
    }
    cudaEventDestroy(e[0]);
    cudaEventDestroy(e[1]);
    if (rc != PPM_OK) return rc;
    TRY(grid_map_f32(ctx, ctx->map_n, ctx->map_r2, best));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->map_cells = best;
    if (best_cells) *best_cells = best;
    if (best_ms) *best_ms = best_t;
    return PPM_OK;
}

// ---------------------------------------------------------------------------
// progressive render
// ---------------------------------------------------------------------------
extern "C" const char *ppm_stage_name(int32_t stage) {
    return stage >= 0 && stage < N_STAGES ? STAGE_NAMES[stage] : "";
}

extern "C" int ppm_set_stage_timing(ppm_ctx *ctx, int32_t on) {
    if (!ctx) return PPM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (on && !ctx->tev_made) {
        for (int i = 0; i < TIMING_SLOTS; i++)
            for (int j = 0; j < 8; j++) CK(cudaEventCreate(&ctx->tev[i][j]));
        for (cudaEvent_t &e : ctx->xev) CK(cudaEventCreate(&e));
        ctx->tev_made = true;
    }
    ctx->timing = on != 0;
    ctx->count_gather = on >= 2;   // level 2 also counts gather candidates / hits
    return PPM_OK;
}

// event slot layout: 0 pass start, 1 after trace+bbox, 2 after map build,
// 7 after joining the eye stream, 3 after gather, 4 after accumulate/end;
// 5/6 eye start/end on the side stream
static int drain_timing(ppm_ctx *ctx) {
    if (ctx->slot_pending == 0) return PPM_OK;
    CK(cudaStreamSynchronize(ctx->s));
    CK(cudaStreamSynchronize(ctx->s2));
    for (int k = 0; k < ctx->slot_pending; k++) {
        int slot = (ctx->slot_head - ctx->slot_pending + k + TIMING_SLOTS) % TIMING_SLOTS;
        cudaEvent_t *e = ctx->tev[slot];
        float ms;
        const int pairs[N_RENDER_STAGES][2] = {{0, 1}, {1, 2}, {5, 6}, {7, 3}, {3, 4}};
        for (int st = 0; st < N_RENDER_STAGES; st++) {
            CK(cudaEventElapsedTime(&ms, e[pairs[st][0]], e[pairs[st][1]]));
            ctx->stage_ms[st] += ms;
            ctx->stage_calls[st] += 1;
        }
    }
    ctx->slot_pending = 0;
    return PPM_OK;
}

static int enqueue_pass(ppm_ctx *ctx, bool capture) {
    const bool mixed = ctx->cfg.precision == PPM_PRECISION_MIXED;
    const int uc = ctx->cfg.use_classic ? 1 : 0;
    cudaStream_t s = ctx->s, s2 = ctx->s2;
    cudaEvent_t *ev = nullptr;
    if (ctx->timing && !capture) {
        if (ctx->slot_pending == TIMING_SLOTS) TRY(drain_timing(ctx));
        ev = ctx->tev[ctx->slot_head];
        ctx->slot_head = (ctx->slot_head + 1) % TIMING_SLOTS;
        ctx->slot_pending++;
    }
    int kernels = 0;
    const int g8 = grid_blocks(ctx, 8), g4 = grid_blocks(ctx, 4);
    if (ev) CK(cudaEventRecord(ev[0], s));
    launch_pass_begin(ctx->st, s); kernels++;
    if (ctx->cfg.flags & PPM_RENDER_CLASSIC) {
        // classic tracer: eye rays only (no photons, no map, no gather); the
        // stage events stay in order so the timing table reads zeros there
        if (ev) CK(cudaEventRecord(ev[5], s));
        if (mixed)
            kernels += enqueue_eye<float>(ctx, as<HitPoint<float>>(ctx->hits_f),
                [&](int l, EyeQueue<float> in, EyeQueue<float> out, unsigned long long qcap, HitPoint<float> *h, int g,
                    cudaStream_t st) {
                    launch_eye_level_f(ctx->sv_f, ctx->cam_f, ctx->cfg.seed, ctx->st, uc, l, in, out, qcap, h,
                                       EyeOut<float>{as<float>(ctx->pass_direct32), as<float>(ctx->pass_gather32)}, g,
                                       st, true);
                }, s);
        else
            kernels += enqueue_eye<double>(ctx, as<HitPoint<double>>(ctx->hits_d),
                [&](int l, EyeQueue<double> in, EyeQueue<double> out, unsigned long long qcap, HitPoint<double> *h,
                    int g, cudaStream_t st) {
                    launch_eye_level_d(ctx->sv_d, ctx->cam_d, ctx->cfg.seed, ctx->st, uc, l, in, out, qcap, h,
                                       EyeOut<double>{as<double>(ctx->pass_img)}, g, st, true);
                }, s);
        if (ev) for (int k : {6, 1, 2, 7, 3}) CK(cudaEventRecord(ev[k], s));
        if (mixed)
            launch_accum_mixed(as<float>(ctx->pass_direct32), as<float>(ctx->pass_gather32), ctx->st, ctx->pw,
                               as<double>(ctx->pass_img), as<double>(ctx->sum_img), 3 * ctx->npx, s);
        else
            launch_accum(as<double>(ctx->pass_img), as<double>(ctx->sum_img), 3 * ctx->npx, s);
        launch_pass_end(ctx->st, s);
        kernels += 2;
        if (ev) CK(cudaEventRecord(ev[4], s));
        CK(cudaGetLastError());
        ctx->kernels_per_pass = kernels;
        return PPM_OK;
    }
    // the eye pass does not depend on the photon map: run it on the side stream
    CK(cudaEventRecord(ctx->ev_fork, s));
    CK(cudaStreamWaitEvent(s2, ctx->ev_fork, 0));
    if (ev) CK(cudaEventRecord(ev[5], s2));
    if (mixed)
        kernels += enqueue_eye<float>(ctx, as<HitPoint<float>>(ctx->hits_f),
            [&](int l, EyeQueue<float> in, EyeQueue<float> out, unsigned long long qcap, HitPoint<float> *h, int g,
                cudaStream_t st) {
                launch_eye_level_f(ctx->sv_f, ctx->cam_f, ctx->cfg.seed, ctx->st, uc, l, in, out, qcap, h,
                                   EyeOut<float>{as<float>(ctx->pass_direct32), as<float>(ctx->pass_gather32)}, g, st);
            }, s2);
    else
        kernels += enqueue_eye<double>(ctx, as<HitPoint<double>>(ctx->hits_d),
            [&](int l, EyeQueue<double> in, EyeQueue<double> out, unsigned long long qcap, HitPoint<double> *h, int g,
                cudaStream_t st) {
                launch_eye_level_d(ctx->sv_d, ctx->cam_d, ctx->cfg.seed, ctx->st, uc, l, in, out, qcap, h,
                                   EyeOut<double>{as<double>(ctx->pass_img)}, g, st);
            }, s2);
    const bool tile = mixed && (ctx->cfg.flags & PPM_RENDER_TILE_GATHER);
    if (tile) {   // hit points into Morton order for the tile gather, still on the eye stream
        launch_hit_sort_f(as<HitPoint<float>>(ctx->hits_f), ctx->st, as<uint32_t>(ctx->hcount),
                          as<uint32_t>(ctx->hblock), as<uint32_t>(ctx->hstart), as<uint2>(ctx->hkeyrank),
                          as<HitPoint<float>>(ctx->hits_sorted), grid_blocks(ctx, 8), s2);
        kernels += kernels_per_hit_sort();
    }
    if (ev) CK(cudaEventRecord(ev[6], s2));
    CK(cudaEventRecord(ctx->ev_join, s2));
    // photons; the pass's grid over the scene's box or the photons' bounds
    const bool box = ctx->render_scene_box;
    if (mixed) {
        PhotonBuf<float> pb{as<float4>(ctx->raw_f), as<float4>(ctx->sorted_f), nullptr};
        kernels += enqueue_photon_trace<float>(ctx, ctx->plan, ctx->cfg.seed, uc, pb, s);
        if (!box) launch_bbox_f(pb, ctx->st, -1, g4, s);
        if (ev) CK(cudaEventRecord(ev[1], s));
        if (!box) launch_grid_setup(ctx->st, -1.0, s);   // box scenes: set up by the trace
        launch_hist_f(pb, ctx->st, -1, as<uint32_t>(ctx->count), as<uint2>(ctx->keyrank), g8, s);
        launch_scan(as<uint32_t>(ctx->count), ctx->st, as<uint32_t>(ctx->block_sums), as<uint32_t>(ctx->start), CELL_CAP, s,
                    grid_blocks(ctx, 8));
        launch_scatter_f(pb, ctx->st, -1, as<uint32_t>(ctx->start), as<uint2>(ctx->keyrank), g8, s);
    } else {
        PhotonBuf<double> pb{as<PhotonD>(ctx->raw_d), as<double4>(ctx->spos), as<double4>(ctx->sdir)};
        kernels += enqueue_photon_trace<double>(ctx, ctx->plan, ctx->cfg.seed, uc, pb, s);
        if (!box) launch_bbox_d(pb, ctx->st, -1, g4, s);
        if (ev) CK(cudaEventRecord(ev[1], s));
        launch_grid_setup(ctx->st, -1.0, s);
        launch_hist_d(pb, ctx->st, -1, as<uint32_t>(ctx->count), as<uint2>(ctx->keyrank), g8, s);
        launch_scan(as<uint32_t>(ctx->count), ctx->st, as<uint32_t>(ctx->block_sums), as<uint32_t>(ctx->start), CELL_CAP, s,
                    grid_blocks(ctx, 8));
        launch_scatter_d(pb, ctx->st, -1, as<uint32_t>(ctx->start), as<uint2>(ctx->keyrank), g8, s);
    }
    // [bounds, grid set-up,] histogram, scan, scatter; the FP64 path sets its
    // grid up in a kernel of its own for box scenes too
    kernels += (box ? (mixed ? 2 : 3) : 4) + kernels_per_scan();
    if (ev) CK(cudaEventRecord(ev[2], s));
    CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
    if (ev) CK(cudaEventRecord(ev[7], s));
    if (mixed) {
        GatherOutF go{as<float>(ctx->pass_gather32), nullptr, ctx->count_gather ? &ctx->st->candidates : nullptr,
                      ctx->gather_dump};
        if (!(ctx->cfg.flags & PPM_RENDER_TILE_GATHER)) {
            launch_gather_f(as<HitPoint<float>>(ctx->hits_f), ctx->st, -1, as<float4>(ctx->sorted_f),
                            as<uint32_t>(ctx->start), ctx->cam.pfilter, go, g8, s);
        } else {
            launch_gather_tile_f(as<HitPoint<float>>(ctx->hits_sorted), ctx->st, as<float4>(ctx->sorted_f),
                                 as<uint32_t>(ctx->start), ctx->cam.pfilter, as<TileItem>(ctx->tile_queue),
                                 ctx->tile_cap, go, grid_blocks(ctx, ctx->tile_blocks), s);
            kernels += kernels_per_tile_gather() - 1;
        }
    } else {
        GatherOutD go{as<double>(ctx->pass_img), nullptr, nullptr};
        launch_gather_d(as<HitPoint<double>>(ctx->hits_d), ctx->st, -1, as<double4>(ctx->spos), as<double4>(ctx->sdir),
                        as<uint32_t>(ctx->start), ctx->pw, ctx->cam.pfilter, 0, go, g8, s);
    }
    kernels++;
    if (ev) CK(cudaEventRecord(ev[3], s));
    if (mixed)
        launch_accum_mixed(as<float>(ctx->pass_direct32), as<float>(ctx->pass_gather32), ctx->st, ctx->pw,
                           as<double>(ctx->pass_img), as<double>(ctx->sum_img), 3 * ctx->npx, s);
    else
        launch_accum(as<double>(ctx->pass_img), as<double>(ctx->sum_img), 3 * ctx->npx, s);
    launch_pass_end(ctx->st, s);
    kernels += 2;
    if (ev) CK(cudaEventRecord(ev[4], s));
    CK(cudaGetLastError());
    ctx->kernels_per_pass = kernels;
    return PPM_OK;
}

static double schedule_r2(const ppm_render_cfg &c, int upto) {
    double r = c.radius0 * c.radius0;
    for (int k = 0; k < upto; k++) {
        double i = (double)(k + c.schedule_offset);
        r = r * ((i + c.alpha) / (i + 1.0));
    }
    return r;
}

// Grid cell autotuner of a render: one untimed and two timed passes with each
// of 1 to MAX_CELL_FACTOR cells per radius at the render's middle pass (the captured pass
// graph, which reads the cell factor from the device state, or eager passes
// without a graph); the faster wins.  The trial passes write
// only buffers that the caller's render then resets (state, pass and sum
// images), so the image does not depend on the trial.
static int tune_cells(ppm_ctx *ctx, const ppm_render_cfg &cfg, long long cap, int &best) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return set_err(ctx, PPM_ERR_CUDA, "event"); }
    const bool timing = ctx->timing;
    ctx->timing = false;
    // trials at the middle pass: its radius is typical of the render (the
    // first pass has the largest radius, where finer cells pay off most)
    const int trial = cfg.first_pass + cfg.passes / 2;
    float best_ms = 1e30f;
    int rc = PPM_OK;
    for (int k = 1; k <= MAX_CELL_FACTOR && rc == PPM_OK; k++) {
        float total = 0.0f;
        for (int rep = 0; rep < 3 && rc == PPM_OK; rep++) {   // one warm-up, two timed passes
            rc = upload_state(ctx, schedule_r2(cfg, trial), trial, cfg.alpha, cfg.schedule_offset, (double)k, cap,
                              ctx->hit_cap, ctx->render_sx, CELL_CAP, ctx->render_scene_box);
            if (rc == PPM_OK && cudaEventRecord(e0, ctx->s) != cudaSuccess) rc = set_err(ctx, PPM_ERR_CUDA, "event");
            if (rc == PPM_OK) {
                if (ctx->graph_exec) {   // time the pass the render will replay
                    if (cudaGraphLaunch(ctx->graph_exec, ctx->s) != cudaSuccess) rc = set_err(ctx, PPM_ERR_CUDA, "graph");
                } else {
                    rc = enqueue_pass(ctx, false);
                }
            }
            if (rc == PPM_OK && cudaEventRecord(e1, ctx->s) != cudaSuccess) rc = set_err(ctx, PPM_ERR_CUDA, "event");
            float ms = 0.0f;
            if (rc == PPM_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                rc = set_err(ctx, PPM_ERR_CUDA, "cell tuner timing");
            if (rep > 0) total += ms;
        }
        if (rc == PPM_OK && total < best_ms) { best_ms = total; best = k; }
    }
    ctx->timing = timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != PPM_OK) return rc;
    CK(cudaMemsetAsync(ctx->sum_img.p, 0, sizeof(double) * 3 * ctx->npx, ctx->s));
    CK(cudaMemsetAsync(ctx->pass_img.p, 0, sizeof(double) * 3 * ctx->npx, ctx->s));
    return PPM_OK;
}

extern "C" int ppm_render_begin(ppm_ctx *ctx, const ppm_render_cfg *cfg) {
    if (!ctx || !cfg) return PPM_ERR_INVALID_ARG;
    if (!ctx->have_scene || !ctx->have_cam || ctx->lights.empty())
        return set_err(ctx, PPM_ERR_NOT_READY, "scene (with lights) and camera must be set first");
    if (cfg->nphoton <= 0 || cfg->passes < 0 || !(cfg->radius0 > 0.0) || cfg->precision < 0 || cfg->precision > 1 ||
        cfg->cell_factor < 0 || cfg->cell_factor > MAX_CELL_FACTOR || cfg->first_pass < 0 ||
        (cfg->flags & ~(PPM_RENDER_TUNE_CELLS | PPM_RENDER_CLASSIC | PPM_RENDER_TILE_GATHER)))
        return set_err(ctx, PPM_ERR_INVALID_ARG, "bad render configuration");
    cudaSetDevice(ctx->device);
    drop_graph(ctx);
    ctx->render_scene_box = ctx->scene_box;
    ctx->cfg = *cfg;
    ctx->pw = make_plan(ctx->lights, cfg->nphoton, ctx->plan);
    long long nem = ctx->plan.first[ctx->plan.n_lights];
    if (nem > 0x7fffffffLL / MAX_TRACE) return set_err(ctx, PPM_ERR_INVALID_ARG, "too many photons per pass");
    long long cap = std::max(1LL, nem * MAX_TRACE);
    ctx->npx = (long long)ctx->cam.xreso * ctx->cam.yreso;
    ctx->hit_cap = ctx->npx * HITS_PER_PIXEL;
    const bool photons = !(cfg->flags & PPM_RENDER_CLASSIC);
    if (cfg->precision == PPM_PRECISION_MIXED) {
        if (photons) TRY(ensure_photons_f(ctx, cap, false));
        TRY(ensure(ctx, ctx->hits_f, sizeof(HitPoint<float>) * ctx->hit_cap));
        TRY(ensure_eye_queues(ctx, ctx->npx, sizeof(float4)));
    } else {
        if (photons) TRY(ensure_photons_d(ctx, cap));
        TRY(ensure(ctx, ctx->hits_d, sizeof(HitPoint<double>) * ctx->hit_cap));
        TRY(ensure_eye_queues(ctx, ctx->npx, sizeof(double4)));
    }
    TRY(ensure(ctx, ctx->pass_img, sizeof(double) * 3 * ctx->npx));
    if (cfg->precision == PPM_PRECISION_MIXED) {
        TRY(ensure(ctx, ctx->pass_direct32, sizeof(float) * 3 * ctx->npx));
        TRY(ensure(ctx, ctx->pass_gather32, sizeof(float) * 3 * ctx->npx));
        if (photons && (cfg->flags & PPM_RENDER_TILE_GATHER)) TRY(ensure_hit_sort(ctx));
    }
    TRY(ensure(ctx, ctx->sum_img, sizeof(double) * 3 * ctx->npx));
    CK(cudaMemsetAsync(ctx->sum_img.p, 0, sizeof(double) * 3 * ctx->npx, ctx->s));
    CK(cudaMemsetAsync(ctx->pass_img.p, 0, sizeof(double) * 3 * ctx->npx, ctx->s));
    int cf = cfg->cell_factor ? cfg->cell_factor : 1;
    TRY(upload_state(ctx, schedule_r2(*cfg, cfg->first_pass), cfg->first_pass, cfg->alpha, cfg->schedule_offset, (double)cf,
                     cap, ctx->hit_cap, ctx->render_sx, CELL_CAP, ctx->render_scene_box));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->cell_factor = cf;
    ctx->passes_done = 0;
    ctx->map_kind = 0;
    for (int i = 0; i < 16; i++) { ctx->stage_ms[i] = 0.0; ctx->stage_calls[i] = 0; }
    ctx->slot_pending = 0;
    if (cfg->use_graph) {
        CK(cudaStreamBeginCapture(ctx->s, cudaStreamCaptureModeThreadLocal));
        int r = enqueue_pass(ctx, true);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->s, &g);
        if (r != PPM_OK) { if (g) cudaGraphDestroy(g); return r; }
        if (e != cudaSuccess) return set_err(ctx, PPM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        ctx->graph = g;
        CK(cudaGraphInstantiate(&ctx->graph_exec, g, 0));
    }
    if ((cfg->flags & PPM_RENDER_TUNE_CELLS) && !(cfg->flags & PPM_RENDER_CLASSIC)) {
        TRY(tune_cells(ctx, *cfg, cap, cf));
        TRY(upload_state(ctx, schedule_r2(*cfg, cfg->first_pass), cfg->first_pass, cfg->alpha, cfg->schedule_offset,
                         (double)cf, cap, ctx->hit_cap, ctx->render_sx, CELL_CAP, ctx->render_scene_box));
        CK(cudaStreamSynchronize(ctx->s));
        ctx->cell_factor = cf;
    }
    ctx->render_ready = true;
    return PPM_OK;
}

extern "C" int ppm_render_step(ppm_ctx *ctx, int32_t npasses) {
    if (!ctx || npasses < 0) return PPM_ERR_INVALID_ARG;
    if (!ctx->render_ready) return set_err(ctx, PPM_ERR_NOT_READY, "ppm_render_begin first");
    cudaSetDevice(ctx->device);
    for (int i = 0; i < npasses; i++) {
        if (ctx->graph_exec && !ctx->timing) {
            CK(cudaGraphLaunch(ctx->graph_exec, ctx->s));
        } else {
            TRY(enqueue_pass(ctx, false));
        }
        ctx->passes_done++;
    }
    return PPM_OK;
}

static int check_overflow(ppm_ctx *ctx, PassState &h) {
    TRY(read_state(ctx, h));
    if (h.overflow & 1u) return set_err(ctx, PPM_ERR_CAPACITY, "photon buffer overflow");
    if (h.overflow & 2u) return set_err(ctx, PPM_ERR_CAPACITY, "hit-point buffer overflow (%d per pixel)", HITS_PER_PIXEL);
    if (h.overflow & 4u) return set_err(ctx, PPM_ERR_CAPACITY, "eye stack overflow");
    return PPM_OK;
}

extern "C" int ppm_render_image(ppm_ctx *ctx, double *image_out) {
    if (!ctx || !image_out) return PPM_ERR_INVALID_ARG;
    if (!ctx->render_ready) return set_err(ctx, PPM_ERR_NOT_READY, "ppm_render_begin first");
    cudaSetDevice(ctx->device);
    PassState h;
    TRY(check_overflow(ctx, h));
    CK(cudaMemcpyAsync(image_out, ctx->sum_img.p, sizeof(double) * 3 * ctx->npx, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (ctx->passes_done > 0) {
        double d = (double)ctx->passes_done;
        for (long long i = 0; i < 3 * ctx->npx; i++) image_out[i] = image_out[i] / d;
    }
    return PPM_OK;
}

extern "C" int ppm_render_pass_image(ppm_ctx *ctx, double *image_out) {
    if (!ctx || !image_out) return PPM_ERR_INVALID_ARG;
    if (!ctx->render_ready) return set_err(ctx, PPM_ERR_NOT_READY, "ppm_render_begin first");
    cudaSetDevice(ctx->device);
    PassState h;
    TRY(check_overflow(ctx, h));
    CK(cudaMemcpyAsync(image_out, ctx->pass_img.p, sizeof(double) * 3 * ctx->npx, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PPM_OK;
}

extern "C" int ppm_render_stats(ppm_ctx *ctx, ppm_stats *out) {
    if (!ctx || !out) return PPM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    std::memset(out, 0, sizeof *out);
    PassState h;
    TRY(read_state(ctx, h));
    TRY(drain_timing(ctx));
    out->photons_emitted = ctx->render_ready ? ctx->plan.first[ctx->plan.n_lights] : 0;
    out->photons_stored = (int64_t)h.n_stored;
    out->hit_points = (int64_t)h.n_hits;
    out->grid_cells = h.grid.ncell;
    out->passes_done = ctx->passes_done;
    out->kernels_per_pass = ctx->kernels_per_pass;
    out->n_stages = N_STAGES;
    out->r2 = h.r2;
    for (int i = 0; i < 16; i++) { out->stage_ms[i] = ctx->stage_ms[i]; out->stage_calls[i] = ctx->stage_calls[i]; }
    out->candidates = (int64_t)h.candidates;
    out->in_radius = (int64_t)h.in_radius;
    out->gather_slots = (int64_t)h.slots;
    out->cell_factor = ctx->cell_factor;
    out->photon_rays = (int64_t)h.photon_rays;
    if (ctx->render_ready) {
        int64_t eye = (int64_t)ctx->cam.xreso * ctx->cam.yreso;
        for (int l = 1; l < MAX_TRACE + 2; l++) eye += (int64_t)h.eq[l];
        out->eye_rays = eye;
    }
    return PPM_OK;
}

// One eager pass with the gather's per-hit-point records on, then the pass's
// photon map, hit points, records and gathered image to the host.
extern "C" int ppm_render_gather_export(ppm_ctx *ctx, ppm_gather_export *ex) {
    if (!ctx || !ex) return PPM_ERR_INVALID_ARG;
    if (!ctx->render_ready) return set_err(ctx, PPM_ERR_NOT_READY, "ppm_render_begin first");
    if (ctx->cfg.precision != PPM_PRECISION_MIXED || (ctx->cfg.flags & PPM_RENDER_CLASSIC))
        return set_err(ctx, PPM_ERR_INVALID_ARG, "the gather export needs a mixed-precision photon-mapping render");
    cudaSetDevice(ctx->device);
    if (!ex->photons) {
        ex->n_photons = ctx->photon_cap_f;
        ex->n_hits = ctx->hit_cap;
        return PPM_OK;
    }
    if (!ex->hits || !ex->sums || !ex->counts || !ex->checksums || !ex->gathered || ex->photon_cap < 0 ||
        ex->hit_cap < 0)
        return set_err(ctx, PPM_ERR_INVALID_ARG, "every export array is required");
    TRY(ensure(ctx, ctx->gdump, sizeof(GatherDump) * (size_t)ctx->hit_cap));
    CK(cudaMemsetAsync(ctx->gdump.p, 0, sizeof(GatherDump) * (size_t)ctx->hit_cap, ctx->s));   // walks add into it
    PassState before;
    TRY(read_state(ctx, before));   // the exported pass's radius and index
    ctx->gather_dump = as<GatherDump>(ctx->gdump);
    const int rc = enqueue_pass(ctx, false);
    ctx->gather_dump = nullptr;
    if (rc != PPM_OK) return rc;
    ctx->passes_done++;
    PassState h;
    TRY(check_overflow(ctx, h));
    const long long np = (long long)std::min<unsigned long long>(h.n_stored, h.photon_cap);
    const long long nh = (long long)std::min<unsigned long long>(h.n_hits, h.hit_cap);
    ex->n_photons = np;
    ex->n_hits = nh;
    ex->radius2 = before.r2;
    ex->photon_power = ctx->pw;
    ex->pass = before.pass;
    ex->pfilter = ctx->cam.pfilter;
    if (np > ex->photon_cap || nh > ex->hit_cap)
        return set_err(ctx, PPM_ERR_CAPACITY, "export needs %lld photons and %lld hit points", np, nh);
    std::vector<GatherDump> rec((size_t)nh);
    if (np) CK(cudaMemcpyAsync(ex->photons, ctx->sorted_f.p, sizeof(float4) * np, cudaMemcpyDeviceToHost, ctx->s));
    if (nh) {
        const DevBuf &hb = (ctx->cfg.flags & PPM_RENDER_TILE_GATHER) ? ctx->hits_sorted : ctx->hits_f;
        CK(cudaMemcpyAsync(ex->hits, hb.p, sizeof(HitPoint<float>) * nh, cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaMemcpyAsync(rec.data(), ctx->gdump.p, sizeof(GatherDump) * nh, cudaMemcpyDeviceToHost, ctx->s));
    }
    CK(cudaMemcpyAsync(ex->gathered, ctx->pass_gather32.p, sizeof(float) * 3 * ctx->npx, cudaMemcpyDeviceToHost,
                       ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    for (long long i = 0; i < nh; i++) {
        for (int c = 0; c < 3; c++) ex->sums[3 * i + c] = rec[i].s[c];
        ex->counts[i] = rec[i].count;
        ex->checksums[i] = rec[i].hash;
    }
    return PPM_OK;
}

extern "C" int ppm_render(ppm_ctx *ctx, const ppm_render_cfg *cfg, double *image_out) {
    if (!ctx || !cfg || !image_out) return PPM_ERR_INVALID_ARG;
    TRY(ppm_render_begin(ctx, cfg));
    TRY(ppm_render_step(ctx, cfg->passes));
    return ppm_render_image(ctx, image_out);
}

// ---------------------------------------------------------------------------
// Batched rendering.  One context per job (scene, camera, buffers, pass
// graph); each pass of the whole batch is one launch of a parent graph whose
// children are the jobs' pass graphs, with no edges between jobs, so the GPU
// runs the jobs' kernels side by side.  Jobs with fewer passes drop out of
// the parent graph when they are done.
// ---------------------------------------------------------------------------
struct ppm_batch {
    int device = 0;
    uint64_t seed = 0;
    std::vector<ppm_ctx *> ctxs;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::string err;
    // staged passes: one launch per stage over every job
    int mode = PPM_BATCH_AUTO;
    int sm_count = 0;
    cudaStream_t s2 = nullptr;                 // the eye stages, beside the photon stages
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    void *jobs_d = nullptr, *offs_d = nullptr, *state_d = nullptr;   // job table, prefixes, counters
    size_t jobs_cap = 0;
    int tile = 0;                              // photons per map work item (0: tune)
    int last_staged = 0, last_tile = 0;
    // AUTO: the mode the first eligible render measured as faster (0: not
    // measured yet, 1: staged, 2: graphs) and its trial times per pass
    int auto_pick = 0;
    double trial_ms[2] = {0.0, 0.0};
};

static int batch_err(ppm_batch *b, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    b->err = buf;
    return code;
}

extern "C" int ppm_batch_create(ppm_batch **out, int device, uint64_t seed) {
    if (!out) return PPM_ERR_INVALID_ARG;
    *out = nullptr;
    ppm_ctx *probe = nullptr;
    int st = ppm_ctx_create(&probe, device, seed);
    if (st != PPM_OK) return st;
    ppm_batch *b = new ppm_batch;
    b->device = device;
    b->seed = seed;
    b->ctxs.push_back(probe);
    b->sm_count = probe->sm_count;
    if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&b->s2, cudaStreamNonBlocking, eye_priority()) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess) {
        ppm_batch_destroy(b);
        return PPM_ERR_CUDA;
    }
    *out = b;
    return PPM_OK;
}

extern "C" int ppm_batch_destroy(ppm_batch *b) {
    if (!b) return PPM_OK;
    cudaSetDevice(b->device);
    if (b->s) cudaStreamSynchronize(b->s);
    if (b->s2) cudaStreamSynchronize(b->s2);
    for (ppm_ctx *c : b->ctxs) ppm_ctx_destroy(c);
    for (void *p : {b->jobs_d, b->offs_d, b->state_d})
        if (p) cudaFree(p);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->s) cudaStreamDestroy(b->s);
    if (b->s2) cudaStreamDestroy(b->s2);
    delete b;
    return PPM_OK;
}

extern "C" int ppm_batch_set_mode(ppm_batch *b, int32_t mode, int32_t tile) {
    if (!b || mode < PPM_BATCH_AUTO || mode > PPM_BATCH_GRAPHS || tile < 0 || tile > (1 << 20))
        return PPM_ERR_INVALID_ARG;
    b->mode = mode;
    b->tile = tile;
    b->auto_pick = 0;
    return PPM_OK;
}

extern "C" int ppm_batch_info(const ppm_batch *b, int32_t *staged, int32_t *tile) {
    if (!b) return PPM_ERR_INVALID_ARG;
    if (staged) *staged = b->last_staged;
    if (tile) *tile = b->last_tile;
    return PPM_OK;
}

extern "C" int ppm_batch_trial_ms(const ppm_batch *b, double *staged_ms, double *graphs_ms) {
    if (!b) return PPM_ERR_INVALID_ARG;
    if (!b->auto_pick) return PPM_ERR_NOT_READY;
    if (staged_ms) *staged_ms = b->trial_ms[0];
    if (graphs_ms) *graphs_ms = b->trial_ms[1];
    return PPM_OK;
}

extern "C" const char *ppm_batch_last_error(const ppm_batch *b) { return b ? b->err.c_str() : ""; }

// ---------------------------------------------------------------------------
// Staged batched passes: every job keeps its own context (scene, camera,
// buffers, pass state, cell tuning), and one pass of the whole batch is one
// launch per stage over all jobs (ppm_batch.cuh): begin, the ten eye levels
// (on a second stream), photon trace, map build (bounds, grid, histogram,
// scan, scatter), gather, accumulate, end -- 22 launches for any number of
// jobs, captured once as a CUDA graph.  Jobs that have rendered all their
// passes leave the table (the graph is captured again for the rest).
// ---------------------------------------------------------------------------
namespace {

// photons per work item of the map-build stages tried by the batch's tuner
const int BATCH_TILES[] = {1024, 4096, 16384};

JobDev job_dev(ppm_ctx *c) {
    JobDev d{};
    d.sv = c->sv_f;
    d.cam = c->cam_f;
    d.plan = c->plan;
    d.st = c->st;
    d.seed = c->cfg.seed;
    d.raw = as<float4>(c->raw_f);
    d.sorted = as<float4>(c->sorted_f);
    d.count = as<uint32_t>(c->count);
    d.start = as<uint32_t>(c->start);
    d.block_sums = as<uint32_t>(c->block_sums);
    d.keyrank = as<uint2>(c->keyrank);
    d.hits = as<HitPoint<float>>(c->hits_f);
    d.qa = EyeQueue<float>{as<float4>(c->eqb[0]), as<float4>(c->eqb[1]), as<float4>(c->eqb[2])};
    d.qb = EyeQueue<float>{as<float4>(c->eqb[3]), as<float4>(c->eqb[4]), as<float4>(c->eqb[5])};
    d.eq_cap = (unsigned long long)c->eq_cap;
    d.direct = as<float>(c->pass_direct32);
    d.gathered = as<float>(c->pass_gather32);
    d.pass_img = as<double>(c->pass_img);
    d.sum_img = as<double>(c->sum_img);
    d.pw = c->pw;
    d.npx = c->npx;
    d.uc = c->cfg.use_classic ? 1 : 0;
    d.pfilter = c->cam.pfilter;
    return d;
}

}  // namespace

// the job table and prefixes of the jobs in `act` to the device (nothing of
// the batch may be running)
static int batch_upload_table(ppm_batch *b, const std::vector<int> &act) {
    const int nj = (int)act.size();
    std::vector<JobDev> tab((size_t)nj);
    std::vector<long long> offs(3 * (size_t)(nj + 1), 0);
    long long *emit = offs.data(), *slots = emit + nj + 1, *px = slots + nj + 1;
    for (int k = 0; k < nj; k++) {
        ppm_ctx *c = b->ctxs[act[k]];
        tab[k] = job_dev(c);
        emit[k + 1] = emit[k] + c->plan.first[c->plan.n_lights];
        slots[k + 1] = slots[k] + eye_slots(c->cam.xreso, c->cam.yreso);
        px[k + 1] = px[k] + 3 * c->npx;
    }
    if (b->jobs_cap < (size_t)nj) {
        for (void **p : {&b->jobs_d, &b->offs_d})
            if (*p) { cudaFree(*p); *p = nullptr; }
        b->jobs_cap = 0;
        if (cudaMalloc(&b->jobs_d, sizeof(JobDev) * nj) != cudaSuccess ||
            cudaMalloc(&b->offs_d, sizeof(long long) * 3 * (nj + 1)) != cudaSuccess)
            return batch_err(b, PPM_ERR_OOM, "no device memory for the job table of %d jobs", nj);
        b->jobs_cap = (size_t)nj;
    }
    if (!b->state_d && cudaMalloc(&b->state_d, sizeof(BatchState)) != cudaSuccess)
        return batch_err(b, PPM_ERR_OOM, "no device memory for the batch counters");
    CK_B(cudaMemcpyAsync(b->jobs_d, tab.data(), sizeof(JobDev) * nj, cudaMemcpyHostToDevice, b->s));
    CK_B(cudaMemcpyAsync(b->offs_d, offs.data(), sizeof(long long) * offs.size(), cudaMemcpyHostToDevice, b->s));
    CK_B(cudaStreamSynchronize(b->s));
    return PPM_OK;
}

// one pass of the jobs in the uploaded table, captured as a graph
static int batch_capture(ppm_batch *b, int nj, int tile, cudaGraphExec_t *exec) {
    const JobDev *jd = static_cast<const JobDev *>(b->jobs_d);
    const long long *emit = static_cast<const long long *>(b->offs_d), *slots = emit + nj + 1, *px = slots + nj + 1;
    BatchState *bs = static_cast<BatchState *>(b->state_d);
    const int sm = b->sm_count;
    CK_B(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
    launch_bt_begin(jd, nj, bs, b->s);
    cudaEventRecord(b->ev_fork, b->s);
    cudaStreamWaitEvent(b->s2, b->ev_fork, 0);
    for (int l = 0; l < MAX_TRACE; l++) launch_bt_eye(jd, nj, l, slots, sm * 4, b->s2);
    cudaEventRecord(b->ev_join, b->s2);
    launch_bt_trace(jd, nj, emit, bs, sm * 3, b->s);
    launch_bt_map(jd, nj, tile, sm * 8, b->s);
    cudaStreamWaitEvent(b->s, b->ev_join, 0);
    launch_bt_gather(jd, nj, bs, sm * 4, b->s);
    launch_bt_accum(jd, nj, px, sm * 8, b->s);
    launch_bt_end(jd, nj, b->s);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->s, &g);
    const cudaError_t le = cudaGetLastError();
    if (e != cudaSuccess || le != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return batch_err(b, PPM_ERR_CUDA, "batch pass capture: %s",
                         cudaGetErrorString(e != cudaSuccess ? e : le));
    }
    const cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return batch_err(b, PPM_ERR_CUDA, "batch pass graph: %s", cudaGetErrorString(ie));
    return PPM_OK;
}

// every job's render begun (buffers, state, cells) with its cell size fixed
static int batch_begin_jobs(ppm_batch *b, const ppm_job *jobs, int njobs, bool first) {
    for (int j = 0; j < njobs; j++) {
        ppm_ctx *c = b->ctxs[j];
        ppm_render_cfg cfg = jobs[j].cfg;
        cfg.use_graph = 0;
        if (!first) {   // keep the cell size the first begin tuned
            cfg.cell_factor = c->cell_factor;
            cfg.flags &= ~PPM_RENDER_TUNE_CELLS;
        }
        int st = PPM_OK;
        if (first) {
            st = ppm_scene_upload(c, jobs[j].objs, jobs[j].n_objs, jobs[j].mats, jobs[j].n_mats, jobs[j].lights,
                                  jobs[j].n_lights);
            if (st == PPM_OK) st = ppm_camera_set(c, jobs[j].cam);
        }
        if (st == PPM_OK) st = ppm_render_begin(c, &cfg);
        if (st != PPM_OK) return batch_err(b, st, "job %d: %s", j, c->err.c_str());
    }
    for (int j = 0; j < njobs; j++) CK_B(cudaStreamSynchronize(b->ctxs[j]->s));
    return PPM_OK;
}

// Tile tuner: one staged pass of the whole batch with each work-item size
// (one untimed, two timed; the jobs must be begun), then every job begun
// again.  Returns the best tile and its time per pass.
static int batch_tune_tile(ppm_batch *b, const ppm_job *jobs, int njobs, int *tile, double *ms_per_pass) {
    std::vector<int> all((size_t)njobs);
    for (int j = 0; j < njobs; j++) all[j] = j;
    TRY(batch_upload_table(b, all));
    float best = 1e30f;
    *tile = BATCH_TILES[0];
    for (int cand : BATCH_TILES) {
        cudaGraphExec_t ex = nullptr;
        TRY(batch_capture(b, njobs, cand, &ex));
        float ms = 0.0f;
        cudaError_t e = cudaGraphLaunch(ex, b->s);
        if (e == cudaSuccess) e = cudaEventRecord(b->e0, b->s);
        for (int r = 0; r < 2 && e == cudaSuccess; r++) e = cudaGraphLaunch(ex, b->s);
        if (e == cudaSuccess) e = cudaEventRecord(b->e1, b->s);
        if (e == cudaSuccess) e = cudaEventSynchronize(b->e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->e0, b->e1);
        cudaGraphExecDestroy(ex);
        if (e != cudaSuccess) return batch_err(b, PPM_ERR_CUDA, "batch tile tuner: %s", cudaGetErrorString(e));
        if (ms < best) { best = ms; *tile = cand; }
    }
    *ms_per_pass = best / 2.0;
    return batch_begin_jobs(b, jobs, njobs, false);
}

// One launch of a parent graph holding every job's own pass graph (the
// jobs in `act`, begun with use_graph) -- one pass of those jobs.
static int batch_parent_graph(ppm_batch *b, const std::vector<int> &act, cudaGraphExec_t *exec) {
    cudaGraph_t parent = nullptr;
    CK_B(cudaGraphCreate(&parent, 0));
    int rc = PPM_OK;
    for (int j : act) {
        cudaGraphNode_t node;
        cudaError_t e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, b->ctxs[j]->graph);
        if (e != cudaSuccess) {
            // name the node types of the job's graph, for the error
            size_t n = 0;
            int types[16] = {0};
            if (cudaGraphGetNodes(b->ctxs[j]->graph, nullptr, &n) == cudaSuccess && n) {
                std::vector<cudaGraphNode_t> nodes(n);
                if (cudaGraphGetNodes(b->ctxs[j]->graph, nodes.data(), &n) == cudaSuccess)
                    for (cudaGraphNode_t nd : nodes) {
                        cudaGraphNodeType t;
                        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && (int)t >= 0 && (int)t < 16) types[(int)t]++;
                    }
            }
            std::string census;
            for (int t = 0; t < 16; t++)
                if (types[t]) census += " type" + std::to_string(t) + "x" + std::to_string(types[t]);
            rc = batch_err(b, PPM_ERR_CUDA, "job %d graph (%zu nodes:%s): %s", j, n, census.c_str(),
                           cudaGetErrorString(e));
            break;
        }
    }
    if (rc == PPM_OK) {
        cudaError_t e = cudaGraphInstantiate(exec, parent, 0);
        if (e != cudaSuccess) rc = batch_err(b, PPM_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
    }
    cudaGraphDestroy(parent);
    return rc;
}

// AUTO's measurement, on the first eligible render of a batch: the staged
// tile tuner's best pass, then one pass of the jobs' graphs side by side
// (one untimed, two timed, the jobs begun with the cells already tuned);
// the faster mode is kept for this and later renders.
static int batch_auto_trial(ppm_batch *b, const ppm_job *jobs, int njobs) {
    TRY(batch_begin_jobs(b, jobs, njobs, true));
    int tile = 0;
    double staged_ms = 0.0;
    TRY(batch_tune_tile(b, jobs, njobs, &tile, &staged_ms));
    std::vector<int> all((size_t)njobs);
    for (int j = 0; j < njobs; j++) {
        all[j] = j;
        ppm_ctx *c = b->ctxs[j];
        ppm_render_cfg cfg = jobs[j].cfg;
        cfg.use_graph = 1;
        cfg.cell_factor = c->cell_factor;
        cfg.flags &= ~PPM_RENDER_TUNE_CELLS;
        int st = ppm_render_begin(c, &cfg);
        if (st != PPM_OK) return batch_err(b, st, "job %d: %s", j, c->err.c_str());
    }
    for (int j = 0; j < njobs; j++) CK_B(cudaStreamSynchronize(b->ctxs[j]->s));
    cudaGraphExec_t ex = nullptr;
    TRY(batch_parent_graph(b, all, &ex));
    float ms = 0.0f;
    cudaError_t e = cudaGraphLaunch(ex, b->s);
    if (e == cudaSuccess) e = cudaEventRecord(b->e0, b->s);
    for (int r = 0; r < 2 && e == cudaSuccess; r++) e = cudaGraphLaunch(ex, b->s);
    if (e == cudaSuccess) e = cudaEventRecord(b->e1, b->s);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->e0, b->e1);
    cudaGraphExecDestroy(ex);
    if (e != cudaSuccess) return batch_err(b, PPM_ERR_CUDA, "batch mode trial: %s", cudaGetErrorString(e));
    b->trial_ms[0] = staged_ms;
    b->trial_ms[1] = ms / 2.0;
    b->auto_pick = staged_ms <= ms / 2.0 ? 1 : 2;
    b->tile = tile;
    return PPM_OK;
}

static int batch_render_staged(ppm_batch *b, const ppm_job *jobs, int njobs, double *device_ms) {
    TRY(batch_begin_jobs(b, jobs, njobs, true));
    int tile = b->tile;
    if (tile == 0) {
        double ms = 0.0;
        TRY(batch_tune_tile(b, jobs, njobs, &tile, &ms));
    }
    int max_passes = 0;
    for (int j = 0; j < njobs; j++) max_passes = std::max(max_passes, jobs[j].cfg.passes);
    CK_B(cudaEventRecord(b->e0, b->s));
    int p = 0;
    while (p < max_passes) {
        // the jobs still rendering, and the pass at which the next one is done
        std::vector<int> act;
        int until = max_passes;
        for (int j = 0; j < njobs; j++)
            if (jobs[j].cfg.passes > p) {
                act.push_back(j);
                until = std::min(until, jobs[j].cfg.passes);
            }
        TRY(batch_upload_table(b, act));
        cudaGraphExec_t ex = nullptr;
        TRY(batch_capture(b, (int)act.size(), tile, &ex));
        int rc = PPM_OK;
        for (; rc == PPM_OK && p < until; p++) {
            cudaError_t e = cudaGraphLaunch(ex, b->s);
            if (e != cudaSuccess) rc = batch_err(b, PPM_ERR_CUDA, "batch pass %d: %s", p, cudaGetErrorString(e));
        }
        CK_B(cudaStreamSynchronize(b->s));   // the table is rewritten for the next set of jobs
        cudaGraphExecDestroy(ex);
        if (rc != PPM_OK) return rc;
    }
    CK_B(cudaEventRecord(b->e1, b->s));
    CK_B(cudaStreamSynchronize(b->s));
    if (device_ms) {
        float ms = 0.0f;
        CK_B(cudaEventElapsedTime(&ms, b->e0, b->e1));
        *device_ms = ms;
    }
    b->last_staged = 1;
    b->last_tile = tile;
    for (int j = 0; j < njobs; j++) {
        ppm_ctx *c = b->ctxs[j];
        c->passes_done = jobs[j].cfg.passes;
        int st = ppm_render_image(c, jobs[j].image_out);
        if (st != PPM_OK) return batch_err(b, st, "job %d: %s", j, c->err.c_str());
    }
    return PPM_OK;
}

extern "C" int ppm_batch_render(ppm_batch *b, const ppm_job *jobs, int32_t njobs, double *device_ms) {
    if (!b || njobs < 0 || (njobs && !jobs)) return PPM_ERR_INVALID_ARG;
    cudaSetDevice(b->device);
    for (int j = 0; j < njobs; j++) {
        const ppm_job &jb = jobs[j];
        if (!jb.cam || !jb.image_out) return batch_err(b, PPM_ERR_INVALID_ARG, "job %d: camera and image are required", j);
    }
    while ((int)b->ctxs.size() < njobs) {
        ppm_ctx *c = nullptr;
        int st = ppm_ctx_create(&c, b->device, b->seed);
        if (st != PPM_OK) return batch_err(b, st, "context for job %zu: %s", b->ctxs.size(), ppm_last_error(nullptr));
        b->ctxs.push_back(c);
    }
    // staged passes need every job to be a mixed-precision photon-mapping
    // render with the default gather
    bool staged = b->mode != PPM_BATCH_GRAPHS && njobs > 0 && njobs <= BATCH_MAX_JOBS;
    for (int j = 0; j < njobs && staged; j++)
        staged = jobs[j].cfg.precision == PPM_PRECISION_MIXED &&
                 !(jobs[j].cfg.flags & (PPM_RENDER_CLASSIC | PPM_RENDER_TILE_GATHER));
    if (b->mode == PPM_BATCH_STAGED && !staged)
        return batch_err(b, PPM_ERR_INVALID_ARG, "staged batch passes take 1 to %d mixed-precision photon-mapping "
                         "jobs with the default gather", BATCH_MAX_JOBS);
    if (staged && b->mode == PPM_BATCH_AUTO) {
        if (!b->auto_pick) TRY(batch_auto_trial(b, jobs, njobs));
        staged = b->auto_pick == 1;
    }
    if (staged) return batch_render_staged(b, jobs, njobs, device_ms);
    b->last_staged = 0;
    b->last_tile = 0;
    int max_passes = 0;
    for (int j = 0; j < njobs; j++) {
        const ppm_job &jb = jobs[j];
        ppm_ctx *c = b->ctxs[j];
        ppm_render_cfg cfg = jb.cfg;
        cfg.use_graph = 1;
        int st = ppm_scene_upload(c, jb.objs, jb.n_objs, jb.mats, jb.n_mats, jb.lights, jb.n_lights);
        if (st == PPM_OK) st = ppm_camera_set(c, jb.cam);
        if (st == PPM_OK) st = ppm_render_begin(c, &cfg);
        if (st != PPM_OK) return batch_err(b, st, "job %d: %s", j, c->err.c_str());
        max_passes = std::max(max_passes, cfg.passes);
    }
    // every job's set-up (uploads, tuning, capture) ran on its own stream
    for (int j = 0; j < njobs; j++) CK_B(cudaStreamSynchronize(b->ctxs[j]->s));
    CK_B(cudaEventRecord(b->e0, b->s));
    int p = 0;
    while (p < max_passes) {
        // jobs still running, and the pass at which the next one finishes
        std::vector<int> act;
        int until = max_passes;
        for (int j = 0; j < njobs; j++)
            if (jobs[j].cfg.passes > p) {
                act.push_back(j);
                until = std::min(until, jobs[j].cfg.passes);
            }
        cudaGraphExec_t exec = nullptr;
        int rc = batch_parent_graph(b, act, &exec);
        for (; rc == PPM_OK && p < until; p++) {
            cudaError_t e = cudaGraphLaunch(exec, b->s);
            if (e != cudaSuccess) rc = batch_err(b, PPM_ERR_CUDA, "batch pass %d: %s", p, cudaGetErrorString(e));
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (rc != PPM_OK) return rc;
    }
    CK_B(cudaEventRecord(b->e1, b->s));
    CK_B(cudaStreamSynchronize(b->s));
    if (device_ms) {
        float ms = 0.0f;
        CK_B(cudaEventElapsedTime(&ms, b->e0, b->e1));
        *device_ms = ms;
    }
    for (int j = 0; j < njobs; j++) {
        ppm_ctx *c = b->ctxs[j];
        c->passes_done = jobs[j].cfg.passes;
        int st = ppm_render_image(c, jobs[j].image_out);
        if (st != PPM_OK) return batch_err(b, st, "job %d: %s", j, c->err.c_str());
    }
    return PPM_OK;
}
