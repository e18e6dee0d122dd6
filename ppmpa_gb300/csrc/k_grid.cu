// k_grid.cu -- pass bookkeeping, grid sizing and the cell-count scan.
//
// Every per-pass parameter lives in device memory (PassState), so one pass
// can be captured once as a CUDA graph and replayed: the PA radius
// recurrence r2_{k+1} = r2_k * ((k+o)+alpha)/((k+o)+1) (util/iterator.rb:33-38)
// runs on the device in FP64 in k_pass_end.
#include "ppm_launch.h"

namespace ppm {

__device__ __forceinline__ void pass_begin_state(PassState *st) {
    st->n_stored = 0;
    st->n_hits = 0;
    st->candidates = 0;
    st->in_radius = 0;
    st->slots = 0;
    st->rows = 0;
    st->gather_next = 0;
    st->tile_items = 0;
    st->tile_next = 0;
    st->emit_next = 0;
    st->trace_done = 0;
    st->photon_rays = 0;
    for (int l = 0; l < MAX_TRACE + 2; l++) st->eq[l] = 0;
    st->inv_pi_r2 = ONE_PI_D / st->r2;
    for (int a = 0; a < 3; a++) {
        // a scene of bounded objects gives the grid its box; otherwise the
        // pass's photons do (k_bbox)
        st->bb_lo[a] = ord_enc(st->scene_box ? st->scene_lo[a] : 1e300);
        st->bb_hi[a] = ord_enc(st->scene_box ? st->scene_hi[a] : -1e300);
        st->hb_lo[a] = ordf_enc(0x7f7fffffu);   // +FLT_MAX
        st->hb_hi[a] = ordf_enc(0xff7fffffu);   // -FLT_MAX
    }
}

// Pass set-up.  With a scene box the bounds the grid spans are the box
// (the photons and hit points lie on the scene's objects), and the pass
// launches no k_bbox; the FP32 photon trace then sets the grid up itself
// (one thread, after its loop), the FP64 path in k_grid_setup after the
// trace.  Photons a rounding step outside the box go to the edge cells,
// which only shrinks their cell distance to any query.
__global__ void k_pass_begin(PassState *st) {
    if (threadIdx.x != 0) return;
    pass_begin_state(st);
}

__global__ void k_grid_setup(PassState *st, double r2_override) {
    grid_dependency_wait();
    if (threadIdx.x != 0) return;
    grid_setup_state(st, r2_override);
    grid_dependents_launch();
}

// Exclusive scan of the per-key counts into start[] (the photon map's cell
// starts) in tiles of SCAN_TILE keys: per-tile sums, a one-block scan of the
// tile sums, then each tile scanned from its offset.  The tile kernels loop
// over the tiles the pass's grid has (nkeys varies per pass; the launch is
// sized once for the capacity), read and write 16 bytes per thread per
// round, and clear the counts for the next pass.
constexpr int SCAN_ROUND = 256 * 4;   // keys per round: 256 threads x one uint4

__device__ __forceinline__ uint4 load_counts(const uint32_t *count, long long i, long long n) {
    if (i + 3 < n) return *reinterpret_cast<const uint4 *>(count + i);
    uint4 v;
    v.x = i < n ? count[i] : 0u;
    v.y = i + 1 < n ? count[i + 1] : 0u;
    v.z = i + 2 < n ? count[i + 2] : 0u;
    v.w = i + 3 < n ? count[i + 3] : 0u;
    return v;
}

// key count of a scan: a fixed one (fixed >= 0), the pass grid's map keys
// (one per cell), or the query sort's (SCAN_QUERY_KEYS: three radius
// classes per cell)
__device__ __forceinline__ long long scan_keys(const PassState *st, long long fixed) {
    return fixed >= 0 ? fixed : (fixed == SCAN_QUERY_KEYS ? 3 * st->grid.ncell : st->grid.nkeys);
}

// the sum of one tile's counts into block_sums[tile]
__device__ __forceinline__ void scan_reduce_tile(const uint32_t *count, long long n, long long tile,
                                                 uint32_t *block_sums, uint32_t *ws) {
    const long long base = tile * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_TILE / SCAN_ROUND; k++) {
        const uint4 v = load_counts(count, base + (long long)k * SCAN_ROUND + 4 * threadIdx.x, n);
        s += (v.x + v.y) + (v.z + v.w);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; w++) t += ws[w];
        block_sums[tile] = t;
    }
    __syncthreads();
}

// exclusive scan of nb <= 4096 tile sums by a block of 1024 threads (the
// batch's per-job scan)
__device__ __forceinline__ void scan_top_block(uint32_t *block_sums, int nb, uint32_t *sh) {
    // each thread owns up to 4 consecutive tile sums
    uint32_t v[4], t = 0;
    for (int j = 0; j < 4; j++) {
        int i = threadIdx.x * 4 + j;
        v[j] = i < nb ? block_sums[i] : 0u;
        t += v[j];
    }
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0u;
        __syncthreads();
        sh[threadIdx.x] += add;
        __syncthreads();
    }
    uint32_t run = sh[threadIdx.x] - t;   // exclusive prefix of this thread's group
    for (int j = 0; j < 4; j++) {
        int i = threadIdx.x * 4 + j;
        if (i < nb) block_sums[i] = run;
        run += v[j];
    }
}

// one tile of the exclusive scan into start[], counts cleared behind it
__device__ __forceinline__ void scan_down_tile(uint32_t *count, long long n, long long tile,
                                               const uint32_t *block_sums, uint32_t *start, uint32_t *ws) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long base = tile * SCAN_TILE;
    uint32_t run = block_sums[tile];   // keys before this tile
#pragma unroll 1
    for (int k = 0; k < SCAN_TILE / SCAN_ROUND; k++) {
        const long long i = base + (long long)k * SCAN_ROUND + 4 * threadIdx.x;
        const uint4 v = load_counts(count, i, n);
        const uint32_t t = (v.x + v.y) + (v.z + v.w);
        uint32_t incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned)o) incl += u;
        }
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        uint32_t woff = 0, total = 0;
#pragma unroll
        for (int w = 0; w < 8; w++) {
            const uint32_t x = ws[w];
            woff += (unsigned)w < warp ? x : 0u;
            total += x;
        }
        uint4 o;
        o.x = run + woff + incl - t;
        o.y = o.x + v.x;
        o.z = o.y + v.y;
        o.w = o.z + v.z;
        if (i + 3 < n) {
            *reinterpret_cast<uint4 *>(start + i) = o;
            *reinterpret_cast<uint4 *>(count + i) = make_uint4(0u, 0u, 0u, 0u);
        } else {
            const uint32_t ov[4] = {o.x, o.y, o.z, o.w};
            for (int j = 0; j < 4; j++)
                if (i + j < n) {
                    start[i + j] = ov[j];
                    count[i + j] = 0u;
                }
        }
        run += total;
        __syncthreads();   // ws is rewritten by the next round
    }
    if (threadIdx.x == 0 && base + SCAN_TILE >= n) start[n] = run;   // the tile holding the last key
}

__global__ void __launch_bounds__(256) k_scan_reduce(const uint32_t *count, const PassState *st, long long fixed,
                                                     uint32_t *block_sums) {
    grid_dependency_wait();
    const long long n = scan_keys(st, fixed);
    const long long ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    __shared__ uint32_t ws[8];
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) scan_reduce_tile(count, n, tile, block_sums, ws);
    grid_dependents_launch();
}

// exclusive scan of nb <= 4096 tile sums by one block of 256 threads, 16
// consecutive sums per thread: warp shuffles and one block barrier
__device__ __forceinline__ void scan_top_256(uint32_t *block_sums, int nb, uint32_t *sh) {
    constexpr int PER = 4096 / 256;
    uint32_t v[PER], t = 0;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int i = threadIdx.x * PER + j;
        v[j] = i < nb ? block_sums[i] : 0u;
        t += v[j];
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += u;
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    uint32_t run = incl - t;
    for (unsigned w = 0; w < warp; w++) run += sh[w];
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int i = threadIdx.x * PER + j;
        if (i < nb) block_sums[i] = run;
        run += v[j];
    }
}

__global__ void __launch_bounds__(256) k_scan_top(uint32_t *block_sums, const PassState *st, long long fixed) {
    grid_dependency_wait();
    const long long n = scan_keys(st, fixed);
    __shared__ uint32_t sh[8];
    scan_top_256(block_sums, (int)((n + SCAN_TILE - 1) / SCAN_TILE), sh);
    grid_dependents_launch();
}

__global__ void __launch_bounds__(256) k_scan_down(uint32_t *count, const PassState *st, long long fixed,
                                                   const uint32_t *block_sums, uint32_t *start) {
    grid_dependency_wait();
    const long long n = scan_keys(st, fixed);
    const long long ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    __shared__ uint32_t ws[8];
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
        scan_down_tile(count, n, tile, block_sums, start, ws);
    grid_dependents_launch();
}

__global__ void k_accum(const double *pass_img, double *sum, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        sum[i] += pass_img[i];
}

__device__ __forceinline__ void pass_end_state(PassState *st) {
    double i = (double)(st->pass + st->offset);
    st->r2 = st->r2 * ((i + st->alpha) / (i + 1.0));
    st->pass += 1;
}

__global__ void k_pass_end(PassState *st) {
    if (threadIdx.x != 0) return;
    pass_end_state(st);
}

// ---- batched passes: per-job bookkeeping and the per-job scan ---------------
__global__ void k_bt_begin(const JobDev *jobs, int njobs, BatchState *bs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) {
        bs->emit_next = 0;
        bs->gather_next = 0;
    }
    if (j < njobs) pass_begin_state(jobs[j].st);
}
__global__ void k_bt_grid(const JobDev *jobs, int njobs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < njobs) grid_setup_state(jobs[j].st, -1.0);
}
__global__ void k_bt_end(const JobDev *jobs, int njobs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < njobs) pass_end_state(jobs[j].st);
}

// work items (job, scan tile) over every job's key counts
__device__ __forceinline__ long long bt_scan_tiles(const JobDev *jobs, int njobs, long long *off) {
    return batch_prefix(off, njobs, [&](int j) { return (jobs[j].st->grid.nkeys + SCAN_TILE - 1) / SCAN_TILE; });
}
__global__ void __launch_bounds__(256) k_bt_scan_reduce(const JobDev *jobs, int njobs) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    __shared__ uint32_t ws[8];
    const long long total = bt_scan_tiles(jobs, njobs, off);
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
        const int j = batch_job(off, njobs, it);
        const JobDev &jd = jobs[j];
        scan_reduce_tile(jd.count, jd.st->grid.nkeys, it - off[j], jd.block_sums, ws);
    }
}
__global__ void __launch_bounds__(1024) k_bt_scan_top(const JobDev *jobs) {   // one block per job
    __shared__ uint32_t sh[1024];
    const JobDev &jd = jobs[blockIdx.x];
    scan_top_block(jd.block_sums, (int)((jd.st->grid.nkeys + SCAN_TILE - 1) / SCAN_TILE), sh);
}
__global__ void __launch_bounds__(256) k_bt_scan_down(const JobDev *jobs, int njobs) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    __shared__ uint32_t ws[8];
    const long long total = bt_scan_tiles(jobs, njobs, off);
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
        const int j = batch_job(off, njobs, it);
        const JobDev &jd = jobs[j];
        scan_down_tile(jd.count, jd.st->grid.nkeys, it - off[j], jd.block_sums, jd.start, ws);
    }
}

void launch_bt_begin(const JobDev *jobs, int njobs, BatchState *bs, cudaStream_t s) {
    k_bt_begin<<<(njobs + 127) / 128, 128, 0, s>>>(jobs, njobs, bs);
}
void launch_bt_grid(const JobDev *jobs, int njobs, cudaStream_t s) {
    k_bt_grid<<<(njobs + 127) / 128, 128, 0, s>>>(jobs, njobs);
}
void launch_bt_end(const JobDev *jobs, int njobs, cudaStream_t s) {
    k_bt_end<<<(njobs + 127) / 128, 128, 0, s>>>(jobs, njobs);
}
void launch_bt_scan(const JobDev *jobs, int njobs, int grid, cudaStream_t s) {
    k_bt_scan_reduce<<<grid, 256, 0, s>>>(jobs, njobs);
    k_bt_scan_top<<<njobs, 1024, 0, s>>>(jobs);
    k_bt_scan_down<<<grid, 256, 0, s>>>(jobs, njobs);
}

void launch_pass_begin(PassState *st, cudaStream_t s) { k_pass_begin<<<1, 32, 0, s>>>(st); }
void launch_grid_setup(PassState *st, double r2_override, cudaStream_t s) {
    launch_pdl(k_grid_setup, dim3(1), dim3(32), s, st, r2_override);
}
void launch_scan(uint32_t *count, const PassState *st, uint32_t *block_sums, uint32_t *start, long long cell_cap,
                 cudaStream_t s, int grid, long long fixed_keys) {
    const long long cap = fixed_keys >= 0 ? fixed_keys : cell_cap;
    const long long tiles = (cap + SCAN_TILE - 1) / SCAN_TILE;
    const int nb = (int)(tiles < grid ? tiles : grid);
    launch_pdl(k_scan_reduce, dim3(nb), dim3(256), s, count, st, fixed_keys, block_sums);
    launch_pdl(k_scan_top, dim3(1), dim3(256), s, block_sums, st, fixed_keys);
    launch_pdl(k_scan_down, dim3(nb), dim3(256), s, count, st, fixed_keys, block_sums, start);
}
int kernels_per_scan() { return 3; }
void launch_accum(const double *pass_img, double *sum, long long n, cudaStream_t s) {
    k_accum<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, s>>>(pass_img, sum, n);
}
void launch_pass_end(PassState *st, cudaStream_t s) { k_pass_end<<<1, 32, 0, s>>>(st); }

// FP32 path: pass image = direct + gathered * pw / (pi r2) in FP64 (the flux
// normalisation by the emitted photon count), added to the FP64 running sum
// (FP64 is a narrow pipe on this GPU: the per-pass constant comes from the
// pass state, computed once at pass begin, and each thread takes several
// elements, so the FP64 work per element is the two conversions, one fused
// multiply-add and the running-sum add.)
// Four elements per thread per step: 16-byte loads of the FP32 images and of
// the running sum, 16-byte stores (the buffers are cudaMalloc'd, so element
// 4q is 16-byte aligned for floats and 32-byte aligned for doubles); the
// last n mod 4 elements one at a time.
__device__ __forceinline__ double accum_one(float d, float g, double kk) { return (double)d + (double)g * kk; }

__global__ void k_accum_mixed(const float *direct, const float *gathered, const PassState *st, double pw,
                              double *pass_img, double *sum, long long n) {
    grid_dependency_wait();
    const double kk = pw * st->inv_pi_r2;
    const long long n4 = n / 4, stride = (long long)gridDim.x * blockDim.x;
    const float4 *d4 = reinterpret_cast<const float4 *>(direct), *g4 = reinterpret_cast<const float4 *>(gathered);
    double2 *p2 = reinterpret_cast<double2 *>(pass_img), *s2 = reinterpret_cast<double2 *>(sum);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
        const float4 d = d4[q], g = g4[q];
        const double2 sa = s2[2 * q], sb = s2[2 * q + 1];
        const double v0 = accum_one(d.x, g.x, kk), v1 = accum_one(d.y, g.y, kk);
        const double v2 = accum_one(d.z, g.z, kk), v3 = accum_one(d.w, g.w, kk);
        p2[2 * q] = make_double2(v0, v1);
        p2[2 * q + 1] = make_double2(v2, v3);
        s2[2 * q] = make_double2(sa.x + v0, sa.y + v1);
        s2[2 * q + 1] = make_double2(sb.x + v2, sb.y + v3);
    }
    for (long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double v = accum_one(direct[i], gathered[i], kk);
        pass_img[i] = v;
        sum[i] += v;
    }
}
void launch_accum_mixed(const float *direct, const float *gathered, const PassState *st, double pw, double *pass_img,
                        double *sum, long long n, cudaStream_t s) {
    const long long q = (n + 3) / 4;
    launch_pdl(k_accum_mixed, dim3((unsigned)((q + 255) / 256 < 1024 ? (q + 255) / 256 : 1024)), dim3(256), s, direct,
               gathered, st, pw, pass_img, sum, n);
}

}  // namespace ppm
