// k_f64.cu -- FP64 (plain) path instantiations.  Built with --fmad=false:
// no multiply-add contraction, so each double expression rounds as written
// and the photon paths match the FP64 host restatement bit for bit.
#define PPM_BUILD_F64 1
#include "ppm_launch.h"

namespace ppm {

void launch_trace_d(const SceneView<double> &sc, const EmitPlan &plan, uint64_t seed, PassState *st, int uc,
                    PhotonBuf<double> photons, int grid, cudaStream_t s) {
    if (sc.bvh)
        k_trace<double, true><<<grid, TRACE_THREADS, 0, s>>>(with_bvh(sc), plan, seed, st, uc, photons);
    else
        k_trace<double, false><<<grid, TRACE_THREADS, 0, s>>>(sc, plan, seed, st, uc, photons);
}
void launch_bbox_d(PhotonBuf<double> buf, PassState *st, long long n_fixed, int grid, cudaStream_t s) {
    launch_pdl(k_bbox<double>, dim3(grid), dim3(256), s, buf, st, n_fixed);
}
void launch_hist_d(PhotonBuf<double> buf, PassState *st, long long n_fixed, uint32_t *count, uint2 *keyrank, int grid,
                   cudaStream_t s) {
    launch_pdl(k_cell_hist<double>, dim3(grid), dim3(256), s, buf, st, n_fixed, count, keyrank);
}
void launch_scatter_d(PhotonBuf<double> buf, PassState *st, long long n_fixed, const uint32_t *start,
                      const uint2 *keyrank, int grid, cudaStream_t s) {
    launch_pdl(k_scatter<double>, dim3(grid), dim3(256), s, buf, st, n_fixed, start, keyrank);
}
void launch_eye_level_d(const SceneView<double> &sc, const DCamera<double> &cam, uint64_t seed, PassState *st, int uc,
                        int level, EyeQueue<double> in, EyeQueue<double> out, unsigned long long qcap,
                        HitPoint<double> *hits, EyeOut<double> pix, int grid, cudaStream_t s, bool classic) {
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
        cudaLaunchKernelEx(&c, k_eye_level_bvh<double, true>, with_bvh(sc), cam, seed, st, uc, level, in, out, qcap, hits, pix);
    else if (sc.bvh)
        cudaLaunchKernelEx(&c, k_eye_level_bvh<double, false>, with_bvh(sc), cam, seed, st, uc, level, in, out, qcap, hits, pix);
    else if (classic)
        cudaLaunchKernelEx(&c, k_eye_level<double, true>, sc, cam, seed, st, uc, level, in, out, qcap, hits, pix);
    else
        cudaLaunchKernelEx(&c, k_eye_level<double, false>, sc, cam, seed, st, uc, level, in, out, qcap, hits, pix);
}
void launch_gather_d(const HitPoint<double> *hits, PassState *st, long long n_fixed, const double4 *spos,
                     const double4 *sdir, const uint32_t *start, double pw, int pfilter, int mode, GatherOutD out,
                     int grid, cudaStream_t s) {
    k_gather_d<<<grid, 256, 0, s>>>(hits, st, n_fixed, spos, sdir, start, pw, pfilter, mode, out);
}
void launch_within_d(const double *q, long long nq, const double *q_r2, const PassState *st, const double4 *smap,
                     const uint32_t *start, unsigned long long *counts, const unsigned long long *offsets,
                     int32_t *idx_out, int grid, cudaStream_t s) {
    k_within<double, double4><<<grid, 256, 0, s>>>(q, nq, q_r2, st, smap, start, nullptr, counts, offsets, idx_out);
}
void launch_make_queries_d(const double *pos, const double *nrm, long long n, HitPoint<double> *hits, cudaStream_t s) {
    if (n <= 0) return;
    k_make_queries<double><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pos, nrm, n, hits);
}
cudaError_t load_estimate_kernels_d() {
    // an attribute query loads a lazily loaded kernel onto the current device
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, k_make_queries<double>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_gather_d);
    return e;
}
void launch_intersect_d(const SceneView<double> &sc, const double *rays, long long n, double *t, int32_t *obj,
                        double *nrm, cudaStream_t s) {
    if (n <= 0) return;
    const unsigned g = (unsigned)((n + 127) / 128);
    if (sc.bvh)
        k_intersect<double, true><<<g, 128, 0, s>>>(with_bvh(sc), rays, n, t, obj, nrm);
    else
        k_intersect<double, false><<<g, 128, 0, s>>>(sc, rays, n, t, obj, nrm);
}

}  // namespace ppm
