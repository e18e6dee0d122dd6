// k_f32.cu -- FP32 mixed-precision path instantiations (FMA contraction on).
// FP64 remains only in the band recheck of the in-radius test, the flux
// normalisation and the image accumulation.
#define PPM_BUILD_F32 1
#include "ppm_launch.h"

namespace ppm {

void launch_trace_f(const SceneView<float> &sc, const EmitPlan &plan, uint64_t seed, PassState *st, int uc,
                    PhotonBuf<float> photons, int grid, cudaStream_t s) {
    if (sc.bvh)
        k_trace<float, true><<<grid, TRACE_THREADS, 0, s>>>(with_bvh(sc), plan, seed, st, uc, photons);
    else
        k_trace<float, false><<<grid, TRACE_THREADS, 0, s>>>(sc, plan, seed, st, uc, photons);
}
void launch_bbox_f(PhotonBuf<float> buf, PassState *st, long long n_fixed, int grid, cudaStream_t s) {
    launch_pdl(k_bbox<float>, dim3(grid), dim3(256), s, buf, st, n_fixed);
}
void launch_hist_f(PhotonBuf<float> buf, PassState *st, long long n_fixed, uint32_t *count, uint2 *keyrank, int grid,
                   cudaStream_t s) {
    launch_pdl(k_cell_hist<float>, dim3(grid), dim3(256), s, buf, st, n_fixed, count, keyrank);
}
void launch_scatter_f(PhotonBuf<float> buf, PassState *st, long long n_fixed, const uint32_t *start,
                      const uint2 *keyrank, int grid, cudaStream_t s) {
    launch_pdl(k_scatter<float>, dim3(grid), dim3(256), s, buf, st, n_fixed, start, keyrank);
}
void launch_eye_level_f(const SceneView<float> &sc, const DCamera<float> &cam, uint64_t seed, PassState *st, int uc,
                        int level, EyeQueue<float> in, EyeQueue<float> out, unsigned long long qcap,
                        HitPoint<float> *hits, EyeOut<float> pix, int grid, cudaStream_t s, bool classic) {
    // levels after 0 launch as programmatic dependents of the level before
    cudaLaunchConfig_t c = {};
    c.gridDim = dim3((unsigned)grid);
    c.blockDim = dim3(128);
    c.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = at;
    c.numAttrs = level > 0 ? 1 : 0;
    if (sc.bvh && classic)
        cudaLaunchKernelEx(&c, k_eye_level_bvh<float, true>, with_bvh(sc), cam, seed, st, uc, level, in, out, qcap, hits, pix);
    else if (sc.bvh)
        cudaLaunchKernelEx(&c, k_eye_level_bvh<float, false>, with_bvh(sc), cam, seed, st, uc, level, in, out, qcap, hits, pix);
    else if (classic)
        cudaLaunchKernelEx(&c, k_eye_level<float, true>, sc, cam, seed, st, uc, level, in, out, qcap, hits, pix);
    else
        cudaLaunchKernelEx(&c, k_eye_level<float, false>, sc, cam, seed, st, uc, level, in, out, qcap, hits, pix);
}
void launch_gather_f(const HitPoint<float> *hits, PassState *st, long long n_fixed, const float4 *smap,
                     const uint32_t *start, int pfilter, GatherOutF out, int grid, cudaStream_t s) {
    if (out.dump)   // the parity export
        launch_pdl(k_gather_f<false, true>, dim3(grid), dim3(256), s, hits, st, n_fixed, smap, start, pfilter, out);
    else if (out.count)
        launch_pdl(k_gather_f<true>, dim3(grid), dim3(256), s, hits, st, n_fixed, smap, start, pfilter, out);
    else
        launch_pdl(k_gather_f<false>, dim3(grid), dim3(256), s, hits, st, n_fixed, smap, start, pfilter, out);
}
void launch_gather_tile_f(const HitPoint<float> *hits, PassState *st, const float4 *smap, const uint32_t *start,
                          int pfilter, TileItem *items, unsigned long long cap, GatherOutF out, int grid,
                          cudaStream_t s) {
    const TileQueue q{items, cap};
#define PPM_TILE(C, D, F)                                                                                   \
    do {                                                                                                    \
        k_gather_tile<C, D, F><<<grid, 32 * GATHER_TILE_WARPS, 0, s>>>(hits, st, smap, start, q, out);       \
        k_gather_tile_items<C, D, F><<<grid, 32 * GATHER_TILE_WARPS, 0, s>>>(hits, st, smap, start, q, out); \
    } while (0)
#define PPM_TILE_F(C, D)                                        \
    do {                                                        \
        if (pfilter == PF_CONE) PPM_TILE(C, D, PF_CONE);        \
        else if (pfilter == PF_GAUSS) PPM_TILE(C, D, PF_GAUSS); \
        else PPM_TILE(C, D, PF_NONE);                           \
    } while (0)
    if (out.dump) PPM_TILE_F(false, true);
    else if (out.count) PPM_TILE_F(true, false);
    else PPM_TILE_F(false, false);
#undef PPM_TILE_F
#undef PPM_TILE
}
void launch_hit_sort_f(const HitPoint<float> *hits, PassState *st, uint32_t *count, uint32_t *block_sums,
                       uint32_t *start, uint2 *keyrank, HitPoint<float> *sorted, int grid, cudaStream_t s) {
    k_hit_bounds<<<grid / 4 > 0 ? grid / 4 : 1, 256, 0, s>>>(hits, st);
    k_hit_key<<<grid, 256, 0, s>>>(hits, st, count, keyrank);
    launch_scan(count, st, block_sums, start, HIT_KEYS, s, grid, HIT_KEYS);
    k_hit_place<<<grid, 256, 0, s>>>(hits, st, keyrank, start, sorted);
}
int kernels_per_hit_sort() { return 3 + kernels_per_scan(); }
int kernels_per_tile_gather() { return 2; }
void launch_estimate_tile_f(const HitPoint<float> *hits, const double *r2s, long long nq, PassState *st,
                            const float4 *smap, const uint32_t *start, double pw, GatherOutF out, int grid,
                            cudaStream_t s) {
    if (nq <= 0) return;
    if (out.count)
        k_estimate_tile<true><<<grid, 32 * GATHER_TILE_WARPS, 0, s>>>(hits, r2s, nq, st, smap, start, pw, out);
    else
        k_estimate_tile<false><<<grid, 32 * GATHER_TILE_WARPS, 0, s>>>(hits, r2s, nq, st, smap, start, pw, out);
}
int estimate_tile_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_estimate_tile<false>, 32 * GATHER_TILE_WARPS, 0) !=
            cudaSuccess || n < 1)
        n = 1;
    return n;
}
int gather_tile_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_gather_tile<false, false, PF_NONE>, 32 * GATHER_TILE_WARPS,
                                                      0) != cudaSuccess || n < 1)
        n = 1;
    return n;
}
void launch_within_f(const float *q, long long nq, const double *q_r2, const PassState *st, const float4 *smap,
                     const uint32_t *start, const int32_t *sidx, unsigned long long *counts,
                     const unsigned long long *offsets, int32_t *idx_out, int grid, cudaStream_t s) {
    k_within<float, float4><<<grid, 256, 0, s>>>(q, nq, q_r2, st, smap, start, sidx, counts, offsets, idx_out);
}
void launch_make_queries_f(const float *pos, const float *nrm, long long n, HitPoint<float> *hits, cudaStream_t s) {
    if (n <= 0) return;
    k_make_queries<float><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pos, nrm, n, hits);
}
void launch_query_sort_f(const float *pos, const float *nrm, const double *r2, long long n, PassState *st,
                         double r2max, uint32_t *count, uint32_t *block_sums, uint32_t *qstart, long long cell_cap,
                         uint2 *keyrank, HitPoint<float> *hits, double *r2_sorted, int grid, cudaStream_t s) {
    if (n <= 0) return;
    // radius classes: r below r_max / 4, below r_max / 2, the rest
    k_query_hist<<<grid, 256, 0, s>>>(pos, r2, n, st, r2max / 16.0, r2max / 4.0, count, keyrank);
    launch_scan(count, st, block_sums, qstart, cell_cap, s, grid, SCAN_QUERY_KEYS);
    k_query_place<<<grid, 256, 0, s>>>(pos, nrm, r2, n, qstart, keyrank, hits, r2_sorted);
}
void launch_intersect_f(const SceneView<float> &sc, const double *rays, long long n, double *t, int32_t *obj,
                        cudaStream_t s) {
    if (n <= 0) return;
    const unsigned g = (unsigned)((n + 127) / 128);
    if (sc.bvh)
        k_intersect<float, true><<<g, 128, 0, s>>>(with_bvh(sc), rays, n, t, obj, nullptr);
    else
        k_intersect<float, false><<<g, 128, 0, s>>>(sc, rays, n, t, obj, nullptr);
}

__global__ void k_pack_photons(const float *pos, const float *dir, const uint8_t *wl, long long n, float4 *raw) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    raw[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2],
                         __uint_as_float(oct_pack(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2], wl[i])));
}
void launch_pack_photons_f(const float *pos, const float *dir, const uint8_t *wl, long long n, float4 *raw,
                           cudaStream_t s) {
    if (n <= 0) return;
    k_pack_photons<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pos, dir, wl, n, raw);
}

}  // namespace ppm

// batched passes over many jobs (the same element bodies)
#include "ppm_batch.cuh"
