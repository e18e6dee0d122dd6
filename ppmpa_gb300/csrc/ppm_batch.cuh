// ppm_batch.cuh -- batched passes: one launch per stage over every job of a
// batch (mixed precision).  Each kernel is the single-job stage's element
// body behind a mapping of flattened work indices to (job, element): a
// prefix of the jobs' counts in shared memory (host-known counts -- emitted
// photons, pixels -- come precomputed; device-known ones -- stored photons,
// queue lengths, hit points -- are summed by each block as it starts).
// Where the body appends with warp-aggregated atomics into one job's
// counters, a job's segment of the flattened space starts on a warp
// boundary (counts padded to 32), so a warp never spans two jobs.
// Included by k_f32.cu (the FP32 unit), whose device functions it uses.
#pragma once
#include "ppm_launch.h"

namespace ppm {

__device__ __forceinline__ long long pad32(long long n) { return (n + 31) & ~31LL; }

__device__ __forceinline__ unsigned long long job_photons(const JobDev &jd) {
    const unsigned long long n = jd.st->n_stored, cap = jd.st->photon_cap;
    return n < cap ? n : cap;
}
__device__ __forceinline__ unsigned long long job_hits(const JobDev &jd) {
    const unsigned long long n = jd.st->n_hits, cap = jd.st->hit_cap;
    return n < cap ? n : cap;
}

// ---------------------------------------------------------------------------
// photon trace: one persistent launch over every job's emitted photons; a
// lane whose photon ended takes the next emission index of the whole batch,
// so lanes of one warp may trace photons of different jobs.  A stored
// photon is appended to its own job's buffer: lanes of one job share one
// atomic (matched by job).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 3) k_bt_trace(const JobDev *jobs, int njobs,
                                                                             const long long *emit_off,
                                                                             BatchState *bs) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    for (int t = threadIdx.x; t <= njobs; t += blockDim.x) off[t] = emit_off[t];
    __syncthreads();
    const unsigned long long n_emit = (unsigned long long)off[njobs];
    const unsigned lane = lane_id();
    PhotonPath<float> ph;
    ph.level = 0;
    int job = 0;
    uint32_t pass = 0;
    bool active = false, exhausted = false;
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !active) & (exhausted ? 0u : 0xffffffffu);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(&bs->emit_next, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + __popc(need) >= n_emit) exhausted = true;
            if (!active) {
                const unsigned long long i = base + __popc(need & ((1u << lane) - 1u));
                if (i < n_emit) {
                    job = batch_job(off, njobs, (long long)i);
                    const JobDev &jd = jobs[job];
                    const long long li = (long long)i - off[job];
                    int l = 0;
                    while (l < jd.plan.n_lights - 1 && li >= jd.plan.first[l + 1]) l++;
                    pass = (uint32_t)jd.st->pass;
                    Rng rg;
                    rg.init<float>(jd.seed, (uint32_t)li, pass, TAG_EMIT);
                    generate_photon(jd.sv.lights[l], rg, ph);
                    ph.item = (uint32_t)li;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) {
            const JobDev &jd = jobs[job];
            const PhotonPath<float> cur = ph;
            bool store, alive;
            V3<float> spos;
            if (jd.sv.bvh) alive = photon_event(with_bvh(jd.sv), jd.seed, pass, jd.uc != 0, ph, store, spos);
            else alive = photon_event(jd.sv, jd.seed, pass, jd.uc != 0, ph, store, spos);
            if (store) {
                const unsigned grp = __match_any_sync(__activemask(), job);
                const int lead = __ffs(grp) - 1;
                unsigned long long slot = 0;
                if ((int)lane == lead) slot = atomicAdd(&jd.st->n_stored, (unsigned long long)__popc(grp));
                slot = __shfl_sync(grp, slot, lead) + __popc(grp & ((1u << lane) - 1u));
                if (slot < jd.st->photon_cap)
                    jd.raw[slot] = make_float4(spos.x, spos.y, spos.z,
                                               __uint_as_float(oct_pack(cur.dir.x, cur.dir.y, cur.dir.z, cur.wl)));
                else
                    atomicOr(&jd.st->overflow, 1u);
            }
            ph.level = cur.level + 1;
            active = alive && ph.level < MAX_TRACE;
        }
    }
}

// ---------------------------------------------------------------------------
// map build: photons in (job, tile) work items of `tile` photons
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long bt_photon_tiles(const JobDev *jobs, int njobs, long long tile, long long *off) {
    return batch_prefix(off, njobs, [&](int j) { return ((long long)job_photons(jobs[j]) + tile - 1) / tile; });
}

__global__ void __launch_bounds__(256) k_bt_bbox(const JobDev *jobs, int njobs, int tile) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    __shared__ float slo[3][8], shi[3][8];
    const long long total = bt_photon_tiles(jobs, njobs, tile, off);
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
        const int j = batch_job(off, njobs, it);
        const JobDev &jd = jobs[j];
        const long long n = (long long)job_photons(jd), b0 = (it - off[j]) * tile;
        const long long b1 = b0 + tile < n ? b0 + tile : n;
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
            const float4 r = jd.raw[i];
            const float v[3] = {r.x, r.y, r.z};
#pragma unroll
            for (int a = 0; a < 3; a++)
                if (v[a] > -1e30f && v[a] < 1e30f) {   // finite and bounded (false for NaN)
                    lo[a] = fminf(lo[a], v[a]);
                    hi[a] = fmaxf(hi[a], v[a]);
                }
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
            for (int o = 16; o > 0; o >>= 1) {
                lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
                hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
            }
            if (lane_id() == 0) { slo[a][threadIdx.x >> 5] = lo[a]; shi[a][threadIdx.x >> 5] = hi[a]; }
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            const int a = threadIdx.x;
            float l = slo[a][0], h = shi[a][0];
            for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
                l = fminf(l, slo[a][w]);
                h = fmaxf(h, shi[a][w]);
            }
            if (l <= h) {
                atomicMin(&jd.st->bb_lo[a], ord_enc((double)l));
                atomicMax(&jd.st->bb_hi[a], ord_enc((double)h));
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_bt_hist(const JobDev *jobs, int njobs, int tile) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    const long long total = bt_photon_tiles(jobs, njobs, tile, off);
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
        const int j = batch_job(off, njobs, it);
        const JobDev &jd = jobs[j];
        const GridParams &g = jd.st->grid;
        const long long n = (long long)job_photons(jd), b0 = (it - off[j]) * tile;
        const long long b1 = b0 + tile < n ? b0 + tile : n;
        for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
            const float4 r = jd.raw[i];
            const uint32_t c = cell_of(g, mk3(r.x, r.y, r.z));
            jd.keyrank[i] = make_uint2(c, atomicAdd(&jd.count[c], 1u));
        }
    }
}

__global__ void __launch_bounds__(256) k_bt_scatter(const JobDev *jobs, int njobs, int tile) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    const long long total = bt_photon_tiles(jobs, njobs, tile, off);
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
        const int j = batch_job(off, njobs, it);
        const JobDev &jd = jobs[j];
        const long long n = (long long)job_photons(jd), b0 = (it - off[j]) * tile;
        const long long b1 = b0 + tile < n ? b0 + tile : n;
        for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
            const uint2 kr = jd.keyrank[i];
            jd.sorted[jd.start[kr.x] + kr.y] = jd.raw[i];
        }
    }
}

// ---------------------------------------------------------------------------
// eye tree: one launch per level over every job's slots (level 0, host
// prefix) or queue (deeper levels), each job's segment padded to 32
// ---------------------------------------------------------------------------
__global__ void __maxnreg__(128) k_bt_eye(const JobDev *jobs, int njobs, int level, const long long *slot_off) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    long long total;
    if (level == 0) {
        for (int t = threadIdx.x; t <= njobs; t += blockDim.x) off[t] = slot_off[t];
        __syncthreads();
        total = off[njobs];
    } else {
        total = batch_prefix(off, njobs, [&](int j) {
            const unsigned long long q = jobs[j].st->eq[level], cap = jobs[j].eq_cap;
            return pad32((long long)(q < cap ? q : cap));
        });
    }
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const int j = batch_job(off, njobs, x);
        const JobDev &jd = jobs[j];
        const unsigned long long i = (unsigned long long)(x - off[j]);
        unsigned long long n;
        if (level == 0) {
            n = (unsigned long long)eye_slots(jd.cam.xreso, jd.cam.yreso);
        } else {
            n = jd.st->eq[level];
            if (n > jd.eq_cap) n = jd.eq_cap;
        }
        if (i >= n) continue;   // padding
        const EyeQueue<float> in = (level & 1) ? jd.qb : jd.qa, out = (level & 1) ? jd.qa : jd.qb;
        const uint32_t pass = (uint32_t)jd.st->pass;
        const unsigned long long hcap = jd.st->hit_cap;
        const long long ntx = eye_tiles_x(jd.cam.xreso);
        const EyeOut<float> pix{jd.direct, jd.gathered};
        if (jd.sv.bvh)
            eye_vertex<float, true, false>(with_bvh(jd.sv), jd.cam, jd.seed, jd.st, jd.uc, level, in, out, jd.eq_cap,
                                           jd.hits, pix, i, pass, hcap, ntx);
        else
            eye_vertex<float, false, false>(jd.sv, jd.cam, jd.seed, jd.st, jd.uc, level, in, out, jd.eq_cap, jd.hits,
                                            pix, i, pass, hcap, ntx);
    }
}

// ---------------------------------------------------------------------------
// gather: the row walk over every job's hit points, two at a time from one
// counter (each job's hit points padded to an even count)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_bt_gather(const JobDev *jobs, int njobs, BatchState *bs) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    const long long total = batch_prefix(off, njobs, [&](int j) { return ((long long)job_hits(jobs[j]) + 1) & ~1LL; });
    const unsigned lane = lane_id();
    for (;;) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(&bs->gather_next, 2ull);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= (unsigned long long)total) break;
        const int j = batch_job(off, njobs, (long long)c);
        const JobDev &jd = jobs[j];
        const unsigned long long qi = c - (unsigned long long)off[j], n = job_hits(jd);
        if (qi >= n) continue;
        const unsigned long long left = n - qi < 2 ? n - qi : 2;
        const GridParams g = jd.st->grid;
        const double r2 = jd.st->r2;
        const GatherOutF go{jd.gathered, nullptr, nullptr, nullptr};
        const unsigned used = gather_step<false, false>(g, r2, jd.hits, qi, left, jd.start, jd.sorted, jd.pfilter, go);
        if (used < left) gather_step<false, false>(g, r2, jd.hits, qi + 1, 1, jd.start, jd.sorted, jd.pfilter, go);
    }
}

// ---------------------------------------------------------------------------
// accumulate: pass image = direct + gathered x pw / (pi r2) in FP64, added
// to the running sum, over every job's pixel channels
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bt_accum(const JobDev *jobs, int njobs, const long long *px_off) {
    __shared__ long long off[BATCH_MAX_JOBS + 1];
    for (int t = threadIdx.x; t <= njobs; t += blockDim.x) off[t] = px_off[t];
    __syncthreads();
    const long long total = off[njobs];
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const int j = batch_job(off, njobs, x);
        const JobDev &jd = jobs[j];
        const long long i = x - off[j];
        const double v = (double)jd.direct[i] + (double)jd.gathered[i] * (jd.pw * jd.st->inv_pi_r2);
        jd.pass_img[i] = v;
        jd.sum_img[i] += v;
    }
}

void launch_bt_trace(const JobDev *jobs, int njobs, const long long *emit_off, BatchState *bs, int grid,
                     cudaStream_t s) {
    k_bt_trace<<<grid, 256, 0, s>>>(jobs, njobs, emit_off, bs);
}
void launch_bt_map(const JobDev *jobs, int njobs, int tile, int grid, cudaStream_t s) {
    k_bt_bbox<<<grid, 256, 0, s>>>(jobs, njobs, tile);
    launch_bt_grid(jobs, njobs, s);
    k_bt_hist<<<grid, 256, 0, s>>>(jobs, njobs, tile);
    launch_bt_scan(jobs, njobs, grid, s);
    k_bt_scatter<<<grid, 256, 0, s>>>(jobs, njobs, tile);
}
void launch_bt_eye(const JobDev *jobs, int njobs, int level, const long long *slot_off, int grid, cudaStream_t s) {
    k_bt_eye<<<grid, 256, 0, s>>>(jobs, njobs, level, slot_off);
}
void launch_bt_gather(const JobDev *jobs, int njobs, BatchState *bs, int grid, cudaStream_t s) {
    k_bt_gather<<<grid, 256, 0, s>>>(jobs, njobs, bs);
}
void launch_bt_accum(const JobDev *jobs, int njobs, const long long *px_off, int grid, cudaStream_t s) {
    k_bt_accum<<<grid, 256, 0, s>>>(jobs, njobs, px_off);
}
int kernels_per_bt_map() { return 4 + kernels_per_scan(); }

}  // namespace ppm
