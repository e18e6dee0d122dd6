// ppm_launch.h -- host-side launch wrappers shared between the translation
// units (k_f64.cu: FP64 path, compiled without FMA contraction; k_f32.cu:
// FP32 mixed path; k_grid.cu: integer grid / scan / pass bookkeeping).
#pragma once
#include <cuda_runtime.h>
#include "ppm_kernels.cuh"

namespace ppm {

// ---- FP64 path -------------------------------------------------------------
// persistent photon tracing: every emitted photon through all its bounces
void launch_trace_d(const SceneView<double> &sc, const EmitPlan &plan, uint64_t seed, PassState *st, int uc,
                    PhotonBuf<double> photons, int grid, cudaStream_t s);
void launch_bbox_d(PhotonBuf<double> buf, PassState *st, long long n_fixed, int grid, cudaStream_t s);
void launch_hist_d(PhotonBuf<double> buf, PassState *st, long long n_fixed, uint32_t *count, uint2 *keyrank, int grid,
                   cudaStream_t s);
void launch_scatter_d(PhotonBuf<double> buf, PassState *st, long long n_fixed, const uint32_t *start,
                      const uint2 *keyrank, int grid, cudaStream_t s);
void launch_eye_level_d(const SceneView<double> &sc, const DCamera<double> &cam, uint64_t seed, PassState *st, int uc,
                        int level, EyeQueue<double> in, EyeQueue<double> out, unsigned long long qcap,
                        HitPoint<double> *hits, EyeOut<double> pix, int grid, cudaStream_t s,
                        bool classic = false);
void launch_gather_d(const HitPoint<double> *hits, PassState *st, long long n_fixed, const double4 *spos,
                     const double4 *sdir, const uint32_t *start, double pw, int pfilter, int mode, GatherOutD out,
                     int grid, cudaStream_t s);
void launch_within_d(const double *q, long long nq, const double *q_r2, const PassState *st, const double4 *smap,
                     const uint32_t *start, unsigned long long *counts, const unsigned long long *offsets,
                     int32_t *idx_out, int grid, cudaStream_t s);
void launch_make_queries_d(const double *pos, const double *nrm, long long n, HitPoint<double> *hits, cudaStream_t s);
// loads the two kernels of the FP64 estimate onto the current device (with
// lazy module loading they would otherwise load at their first launch)
cudaError_t load_estimate_kernels_d();
void launch_intersect_d(const SceneView<double> &sc, const double *rays, long long n, double *t, int32_t *obj,
                        double *nrm, cudaStream_t s);

// ---- FP32 mixed path ---------------------------------------------------------
// persistent photon tracing: every emitted photon through all its bounces
void launch_trace_f(const SceneView<float> &sc, const EmitPlan &plan, uint64_t seed, PassState *st, int uc,
                    PhotonBuf<float> photons, int grid, cudaStream_t s);
void launch_bbox_f(PhotonBuf<float> buf, PassState *st, long long n_fixed, int grid, cudaStream_t s);
void launch_hist_f(PhotonBuf<float> buf, PassState *st, long long n_fixed, uint32_t *count, uint2 *keyrank, int grid,
                   cudaStream_t s);
void launch_scatter_f(PhotonBuf<float> buf, PassState *st, long long n_fixed, const uint32_t *start,
                      const uint2 *keyrank, int grid, cudaStream_t s);
void launch_eye_level_f(const SceneView<float> &sc, const DCamera<float> &cam, uint64_t seed, PassState *st, int uc,
                        int level, EyeQueue<float> in, EyeQueue<float> out, unsigned long long qcap,
                        HitPoint<float> *hits, EyeOut<float> pix, int grid, cudaStream_t s,
                        bool classic = false);
// the render gather, row-walk form (k_gather_f): out.count / out.dump select
// the counting and the parity-export variants
void launch_gather_f(const HitPoint<float> *hits, PassState *st, long long n_fixed, const float4 *smap,
                     const uint32_t *start, int pfilter, GatherOutF out, int grid, cudaStream_t s);
// the render gather, tile form (k_gather_tile, then k_gather_tile_items for
// the queued parts of long walks): 32 hit points per warp; out.count /
// out.dump select the counting and the parity-export variants (the export
// records must be zeroed first); items holds cap queue entries
void launch_gather_tile_f(const HitPoint<float> *hits, PassState *st, const float4 *smap, const uint32_t *start,
                          int pfilter, TileItem *items, unsigned long long cap, GatherOutF out, int grid,
                          cudaStream_t s);
int kernels_per_tile_gather();
// resident blocks per SM of the tile gather (its persistent grid is this x SMs)
int gather_tile_blocks_per_sm();
int estimate_tile_blocks_per_sm();
// the hit points counting-sorted into Morton order of a 128^3 grid over their
// bounds (k_hit_bounds, k_hit_key, scan of HIT_KEYS counts, k_hit_place);
// count must hold HIT_KEYS zeros (the scan leaves it zeroed again)
void launch_hit_sort_f(const HitPoint<float> *hits, PassState *st, uint32_t *count, uint32_t *block_sums,
                       uint32_t *start, uint2 *keyrank, HitPoint<float> *sorted, int grid, cudaStream_t s);
int kernels_per_hit_sort();
void launch_within_f(const float *q, long long nq, const double *q_r2, const PassState *st, const float4 *smap,
                     const uint32_t *start, const int32_t *sidx, unsigned long long *counts,
                     const unsigned long long *offsets, int32_t *idx_out, int grid, cudaStream_t s);
void launch_make_queries_f(const float *pos, const float *nrm, long long n, HitPoint<float> *hits, cudaStream_t s);
// sorts estimate queries by map cell (count -> scan -> place); count is left zeroed
// (key: the map cell and a radius class from r2max)
void launch_query_sort_f(const float *pos, const float *nrm, const double *r2, long long n, PassState *st,
                         double r2max, uint32_t *count, uint32_t *block_sums, uint32_t *qstart, long long cell_cap,
                         uint2 *keyrank, HitPoint<float> *hits, double *r2_sorted, int grid, cudaStream_t s);
// the estimate entry point's gather over the sorted queries (k_estimate_tile)
void launch_estimate_tile_f(const HitPoint<float> *hits, const double *r2s, long long nq, PassState *st,
                            const float4 *smap, const uint32_t *start, double pw, GatherOutF out, int grid,
                            cudaStream_t s);
void launch_intersect_f(const SceneView<float> &sc, const double *rays, long long n, double *t, int32_t *obj,
                        cudaStream_t s);
void launch_pack_photons_f(const float *pos, const float *dir, const uint8_t *wl, long long n, float4 *raw,
                           cudaStream_t s);

// ---- BVH over the bounded objects (k_bvh.cu) --------------------------------------
// 32-bit words of device scratch launch_bvh_build needs for m objects
int bvh_scratch_words(int m, int n_objs);
// builds the internal nodes (at most m - 1) over objs[bounded[0..m)] with
// leaves of at most leaf_max (1..8) objects and the Morton-ordered object
// list `order`; returns the root (0, or a leaf when m <= leaf_max)
int launch_bvh_build(const DObject<double> *objs, const int32_t *bounded, int m, int n_objs, int leaf_max,
                     BvhNode *nodes, int32_t *order, uint32_t *scratch, cudaStream_t s);

// A launch that may begin before the previous kernel in the stream ends
// (programmatic dependent launch): the kernel waits (griddepcontrol.wait)
// before it reads what that kernel wrote, and the previous kernel's blocks
// signal when their work is done, so a chain of dependent launches loses
// no launch latency between its kernels.
template <typename... K, typename... A>
inline void launch_pdl(void (*kernel)(K...), dim3 grid, dim3 block, cudaStream_t s, A &&...args) {
    cudaLaunchConfig_t c = {};
    c.gridDim = grid;
    c.blockDim = block;
    c.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = at;
    c.numAttrs = 1;
    cudaLaunchKernelEx(&c, kernel, std::forward<A>(args)...);
}

// ---- grid / scan / pass bookkeeping ------------------------------------------------
constexpr int SCAN_TILE = 4096;
void launch_pass_begin(PassState *st, cudaStream_t s);
void launch_grid_setup(PassState *st, double r2_override, cudaStream_t s);
// grid: blocks of the two tile kernels (each loops over the pass's tiles)
// fixed_keys >= 0: scan that many keys instead of the pass grid's map keys;
// SCAN_QUERY_KEYS: the query sort's three radius classes per cell.  At most
// 4096 * SCAN_TILE keys: k_scan_top holds 4096 tile sums.
constexpr long long SCAN_QUERY_KEYS = -2;
void launch_scan(uint32_t *count, const PassState *st, uint32_t *block_sums, uint32_t *start, long long cell_cap,
                 cudaStream_t s, int grid, long long fixed_keys = -1);
void launch_accum(const double *pass_img, double *sum, long long n, cudaStream_t s);
void launch_accum_mixed(const float *direct, const float *gathered, const PassState *st, double pw, double *pass_img,
                        double *sum, long long n, cudaStream_t s);
void launch_pass_end(PassState *st, cudaStream_t s);
int kernels_per_scan();

// ---- batched passes (ppm_batch.cuh in k_f32.cu; per-job bookkeeping and scan in k_grid.cu) ----
// one launch per stage over every job of the table (njobs <= BATCH_MAX_JOBS);
// tile is the photons per work item of the map-build stages
void launch_bt_begin(const JobDev *jobs, int njobs, BatchState *bs, cudaStream_t s);
void launch_bt_grid(const JobDev *jobs, int njobs, cudaStream_t s);
void launch_bt_end(const JobDev *jobs, int njobs, cudaStream_t s);
void launch_bt_scan(const JobDev *jobs, int njobs, int grid, cudaStream_t s);
void launch_bt_trace(const JobDev *jobs, int njobs, const long long *emit_off, BatchState *bs, int grid,
                     cudaStream_t s);
void launch_bt_map(const JobDev *jobs, int njobs, int tile, int grid, cudaStream_t s);
void launch_bt_eye(const JobDev *jobs, int njobs, int level, const long long *slot_off, int grid, cudaStream_t s);
void launch_bt_gather(const JobDev *jobs, int njobs, BatchState *bs, int grid, cudaStream_t s);
void launch_bt_accum(const JobDev *jobs, int njobs, const long long *px_off, int grid, cudaStream_t s);
int kernels_per_bt_map();

}  // namespace ppm
