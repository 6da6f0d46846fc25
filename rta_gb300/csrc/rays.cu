// rays.cu -- camera rays, intersection reset and the diffuse bounce pass.
//
//   k_shirley   setup_shirley_rays (librta/cuda-kernels.cu:50-112), the
//               reference's arithmetic through explicit IEEE intrinsics
//   k_reset     reset_intersections (librta/cuda-kernels.cu:24-44)
//   k_bounce    one cosine-weighted diffuse bounce ray per hit (no reference
//               counterpart), compacted in primary-ray order by a single-pass
//               scan with decoupled look-back
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda.h>

#include "bounce.cuh"

namespace rta {

int trace_impl(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt,
               uint32_t nrays, const uint32_t *d_nrays, void *hits, uint32_t mode, uint32_t *stats,
               uint32_t *queue, cudaStream_t s);
int trace_frame_fused(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt, uint32_t nrays,
                      void *hits, uint32_t seed, float eps, float *b_orig, float *b_dir, void *b_hits,
                      uint32_t *b_flag, uint32_t *b_tile, uint32_t *queue, cudaStream_t s);

__global__ void k_shirley(float *__restrict__ dirs, float *__restrict__ orgs, float *__restrict__ maxts,
                          float height, float aspect, int w, int h, V3 vd, V3 pos, V3 up, float maxt)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t id = (size_t)y * w + x;
    orgs[3 * id + 0] = pos.x;
    orgs[3 * id + 1] = pos.y;
    orgs[3 * id + 2] = pos.z;
    maxts[id] = maxt;
    const float width = __fmul_rn(aspect, height);
    float u_s = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn((float)x, 0.5f), (float)w), 2.0f), 1.0f);
    float v_s = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn((float)y, 0.5f), (float)h), 2.0f), 1.0f);
    u_s = __fmul_rn(width, u_s);
    v_s = __fmul_rn(height, v_s);
    V3 W = v_div(vd, v_len(vd));
    V3 TxW = v_cross(up, W);
    V3 U = v_div(TxW, v_len(TxW));
    V3 V = v_cross(W, U);
    V3 dir = v_mul(U, u_s);
    V3 tmp = v_mul(V, v_s);
    dir = v_add(dir, tmp);
    dir = v_add(dir, W);
    dir = v_div(dir, v_len(dir));
    dirs[3 * id + 0] = dir.x;
    dirs[3 * id + 1] = dir.y;
    dirs[3 * id + 2] = dir.z;
}

__global__ void k_reset(HitRec *__restrict__ hits, uint32_t n, const uint32_t *__restrict__ d_n)
{
    const uint32_t cnt = d_n ? *d_n : n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        hits[i].t = FLT_MAX;
        hits[i].beta = 1.0f;
        hits[i].gamma = 2.0f;
    }
}

// ---- diffuse bounce ---- //

constexpr int kBounceThreads = 256;
constexpr int kBounceItems = 4;
constexpr int kBounceTile = kBounceThreads * kBounceItems;
static_assert(kBounceTile == 1 << kBounceTileLog2, "bounce tile");

struct FrameState {
    uint32_t tile_ctr;
    uint32_t count;
    uint32_t queue;
    uint32_t status;
};
// the allocation-free bounce keeps a FrameState in the first 4 words of its scratch
static_assert(sizeof(FrameState) == 16, "FrameState is four 32-bit words");

__global__ void __launch_bounds__(kBounceThreads)
k_bounce(const TriRec *__restrict__ tris, const float *__restrict__ orig, const float *__restrict__ dir,
         const HitRec *__restrict__ hits, uint32_t nrays, uint32_t seed, float eps,
         float *__restrict__ oo, float *__restrict__ od, float *__restrict__ om,
         uint32_t *__restrict__ osrc, uint32_t *__restrict__ tstat, FrameState *__restrict__ fs,
         uint32_t n_tris)
{
    constexpr int kWarps = kBounceThreads / 32;
    constexpr int kChunks = kBounceItems * kWarps;   // 32-ray chunks of a tile, in ray order
    static_assert(kChunks <= 32, "one warp scans the chunk counts");
    __shared__ uint32_t s_tile, s_cnt[kChunks], s_base;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(&fs->tile_ctr, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t ntiles = (nrays + kBounceTile - 1) / kBounceTile;
    // striped arrangement: item k of thread tid is ray tile*TILE + k*THREADS + tid,
    // so every load of a warp is one contiguous run; chunk (k, w) = 32 rays in order
    const uint32_t first = tile * kBounceTile + tid;
    const uint32_t lt_mask = (1u << lane) - 1u;
    bool hit[kBounceItems];
    uint32_t bal[kBounceItems];
#pragma unroll
    for (int k = 0; k < kBounceItems; ++k) {
        const uint32_t i = first + (uint32_t)k * kBounceThreads;
        bool h = false;
        if (i < nrays) {
            const HitRec hr = hits[i];
            h = hr.t != FLT_MAX && hr.ref < n_tris;
        }
        hit[k] = h;
        bal[k] = __ballot_sync(0xffffffffu, h);
        if (lane == 0) s_cnt[k * kWarps + w] = __popc(bal[k]);
    }
    __syncthreads();
    if (w == 0) {
        // exclusive scan of the chunk counts in ray order, then the tile's look-back
        const uint32_t c = lane < kChunks ? s_cnt[lane] : 0u;
        uint32_t x = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane < kChunks) s_cnt[lane] = x - c;
        const uint32_t run = __shfl_sync(0xffffffffu, x, 31);
        if (lane == 0) {
            uint32_t *my = tstat + tile;
            uint32_t excl = 0;
            if (tile == 0) {
                st_volatile(my, kStatPrefix | run);
            } else {
                st_volatile(my, kStatAggregate | run);
                excl = lookback(tstat, 1, tile, &fs->status);
                __threadfence();
                st_volatile(my, kStatPrefix | ((excl + run) & kStatValue));
            }
            s_base = excl;
            if (tile == ntiles - 1) fs->count = excl + run;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBounceItems; ++k) {
        if (!hit[k]) continue;
        const uint32_t i = first + (uint32_t)k * kBounceThreads;
        const uint32_t pos = s_base + s_cnt[k * kWarps + w] + __popc(bal[k] & lt_mask);
        const HitRec hr = hits[i];
        const float o[3] = {orig[3 * (size_t)i], orig[3 * (size_t)i + 1], orig[3 * (size_t)i + 2]};
        const float d[3] = {dir[3 * (size_t)i], dir[3 * (size_t)i + 1], dir[3 * (size_t)i + 2]};
        float bo[3], bd[3];
        bounce_ray(tris[hr.ref], o, d, hr.t, i, seed, eps, bo, bd);
        od[3 * (size_t)pos + 0] = bd[0];
        od[3 * (size_t)pos + 1] = bd[1];
        od[3 * (size_t)pos + 2] = bd[2];
        oo[3 * (size_t)pos + 0] = bo[0];
        oo[3 * (size_t)pos + 1] = bo[1];
        oo[3 * (size_t)pos + 2] = bo[2];
        om[pos] = FLT_MAX;
        osrc[pos] = i;
    }
}

} // namespace rta

using namespace rta;

// The fused frame's bounce rays and hits, gathered from the per-primary-ray
// slots into the frame's buffers in primary-ray order (bounce ray k = the k-th
// flagged ray).  The trace kernel counted each tile's flagged rays
// (tile_cnt), so a tile's first output position is the sum of the counts
// before it: no look-back between tiles.
__global__ void __launch_bounds__(kBounceThreads)
k_bounce_gather(const uint32_t *__restrict__ flag, const float *__restrict__ s_orig,
                const float *__restrict__ s_dir, const HitRec *__restrict__ s_hits, uint32_t nrays,
                float *__restrict__ oo, float *__restrict__ od, float *__restrict__ om, uint32_t *__restrict__ osrc,
                HitRec *__restrict__ ohits, const uint32_t *__restrict__ tile_cnt, FrameState *__restrict__ fs)
{
    constexpr int kWarps = kBounceThreads / 32;
    constexpr int kChunks = kBounceItems * kWarps;
    __shared__ uint32_t s_cnt[kChunks], s_part[kWarps], s_base;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t tile = blockIdx.x;
    const uint32_t ntiles = (nrays + kBounceTile - 1) / kBounceTile;
    const uint32_t first = tile * kBounceTile + tid;
    const uint32_t lt_mask = (1u << lane) - 1u;
    // the tiles before this one
    uint32_t before = 0;
    for (uint32_t q = tid; q < tile; q += kBounceThreads) before += tile_cnt[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) before += __shfl_xor_sync(0xffffffffu, before, off);
    if (lane == 0) s_part[w] = before;
    bool hit[kBounceItems];
    uint32_t bal[kBounceItems];
#pragma unroll
    for (int k = 0; k < kBounceItems; ++k) {
        const uint32_t i = first + (uint32_t)k * kBounceThreads;
        hit[k] = i < nrays && flag[i] != 0u;
        bal[k] = __ballot_sync(0xffffffffu, hit[k]);
        if (lane == 0) s_cnt[k * kWarps + w] = __popc(bal[k]);
    }
    __syncthreads();
    if (w == 0) {
        const uint32_t c = lane < kChunks ? s_cnt[lane] : 0u;
        uint32_t x = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane < kChunks) s_cnt[lane] = x - c;
        const uint32_t run = __shfl_sync(0xffffffffu, x, 31);
        if (lane == 0) {
            uint32_t excl = 0;
            for (int q = 0; q < kWarps; ++q) excl += s_part[q];
            s_base = excl;
            if (tile == ntiles - 1) fs->count = excl + run;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBounceItems; ++k) {
        if (!hit[k]) continue;
        const uint32_t i = first + (uint32_t)k * kBounceThreads;
        const uint32_t pos = s_base + s_cnt[k * kWarps + w] + __popc(bal[k] & lt_mask);
        oo[3 * (size_t)pos + 0] = s_orig[3 * (size_t)i + 0];
        oo[3 * (size_t)pos + 1] = s_orig[3 * (size_t)i + 1];
        oo[3 * (size_t)pos + 2] = s_orig[3 * (size_t)i + 2];
        od[3 * (size_t)pos + 0] = s_dir[3 * (size_t)i + 0];
        od[3 * (size_t)pos + 1] = s_dir[3 * (size_t)i + 1];
        od[3 * (size_t)pos + 2] = s_dir[3 * (size_t)i + 2];
        om[pos] = FLT_MAX;
        osrc[pos] = i;
        ohits[pos] = s_hits[i];
    }
}

struct rta_frame_ctx {
    uint32_t cap = 0;
    float *orig = nullptr, *dir = nullptr, *maxt = nullptr;
    uint32_t *src = nullptr;
    HitRec *hits = nullptr;
    uint32_t *tstat = nullptr;
    FrameState *fs = nullptr;
    // per-primary-ray slots of the fused frame: bounce ray, its hit, a flag
    float *s_orig = nullptr, *s_dir = nullptr;
    HitRec *s_hits = nullptr;
    uint32_t *s_flag = nullptr;
    // optional events around the frame's trace work (rta_frame_set_timing)
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    bool timing = false, timed = false;
};

extern "C" {

int rta_setup_shirley_rays(float *dirs, float *orgs, float *maxts, float tan_half_fovy, float aspect,
                           int w, int h, const float view_dir[3], const float pos[3],
                           const float up[3], float maxt, rta_stream_t stream)
{
    if (!dirs || !orgs || !maxts || !view_dir || !pos || !up || w <= 0 || h <= 0) return RTA_ERR_INVALID;
    dim3 threads(16, 16);
    dim3 blocks((w + 15) / 16, (h + 15) / 16);
    k_shirley<<<blocks, threads, 0, (cudaStream_t)stream>>>(
        dirs, orgs, maxts, tan_half_fovy, aspect, w, h, V3{view_dir[0], view_dir[1], view_dir[2]},
        V3{pos[0], pos[1], pos[2]}, V3{up[0], up[1], up[2]}, maxt);
    return check_launch("k_shirley");
}

int rta_reset_intersections(void *hits, uint32_t w, uint32_t h, rta_stream_t stream)
{
    if (!hits || w == 0 || h == 0) return RTA_ERR_INVALID;
    const uint32_t n = w * h;
    const uint32_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    k_reset<<<blocks, 256, 0, (cudaStream_t)stream>>>((HitRec *)hits, n, nullptr);
    return check_launch("k_reset");
}

int rta_frame_create(rta_frame_ctx **out, uint32_t max_rays)
{
    if (!out || max_rays == 0) return RTA_ERR_INVALID;
    rta_frame_ctx *c = new rta_frame_ctx();
    c->cap = max_rays;
    const uint32_t tiles = (max_rays + kBounceTile - 1) / kBounceTile;
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&c->orig, (size_t)max_rays * 12);
    e = e ? e : cudaMalloc(&c->dir, (size_t)max_rays * 12);
    e = e ? e : cudaMalloc(&c->maxt, (size_t)max_rays * 4);
    e = e ? e : cudaMalloc(&c->src, (size_t)max_rays * 4);
    e = e ? e : cudaMalloc(&c->hits, (size_t)max_rays * sizeof(HitRec));
    e = e ? e : cudaMalloc(&c->tstat, (size_t)tiles * 4);
    e = e ? e : cudaMalloc(&c->fs, sizeof(FrameState));
    e = e ? e : cudaMalloc(&c->s_orig, (size_t)max_rays * 12);
    e = e ? e : cudaMalloc(&c->s_dir, (size_t)max_rays * 12);
    e = e ? e : cudaMalloc(&c->s_hits, (size_t)max_rays * sizeof(HitRec));
    e = e ? e : cudaMalloc(&c->s_flag, (size_t)max_rays * 4);
    e = e ? e : cudaMemset(c->fs, 0, sizeof(FrameState));
    if (e != cudaSuccess) {
        set_cuda_error(e, "rta_frame_create");
        rta_frame_destroy(c);
        return e == cudaErrorMemoryAllocation ? RTA_ERR_NOMEM : RTA_ERR_CUDA;
    }
    *out = c;
    return RTA_OK;
}

int rta_frame_destroy(rta_frame_ctx *c)
{
    if (!c) return RTA_ERR_INVALID;
    if (c->ev_begin) cudaEventDestroy(c->ev_begin);
    if (c->ev_end) cudaEventDestroy(c->ev_end);
    void *ptrs[] = {c->orig, c->dir, c->maxt, c->src, c->hits, c->tstat, c->fs,
                    c->s_orig, c->s_dir, c->s_hits, c->s_flag};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete c;
    return RTA_OK;
}

int rta_frame_get(const rta_frame_ctx *c, rta_frame *out)
{
    if (!c || !out) return RTA_ERR_INVALID;
    out->orig = c->orig;
    out->dir = c->dir;
    out->maxt = c->maxt;
    out->src = c->src;
    out->hits = c->hits;
    out->count = &c->fs->count;
    out->capacity = c->cap;
    return RTA_OK;
}

int rta_diffuse_bounce(rta_frame_ctx *c, const rta_lbvh *bvh, const float *orig, const float *dir,
                       const void *hits, uint32_t nrays, uint32_t seed, float eps,
                       rta_stream_t stream)
{
    if (!c || !bvh || !orig || !dir || !hits || nrays == 0 || nrays > c->cap) return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t tiles = (nrays + kBounceTile - 1) / kBounceTile;
    RTA_CUDA_TRY(cudaMemsetAsync(c->tstat, 0, (size_t)tiles * 4, s));
    RTA_CUDA_TRY(cudaMemsetAsync(&c->fs->tile_ctr, 0, 4, s));
    k_bounce<<<tiles, kBounceThreads, 0, s>>>((const TriRec *)bvh->tris, orig, dir,
                                              (const HitRec *)hits, nrays, seed, eps, c->orig,
                                              c->dir, c->maxt, c->src, c->tstat, c->fs, bvh->n);
    return check_launch("k_bounce");
}

int rta_frame_run(rta_frame_ctx *c, const rta_lbvh *bvh, const float *orig, const float *dir,
                  const float *maxt, uint32_t nrays, void *hits, uint32_t mode, uint32_t seed,
                  float eps, rta_stream_t stream)
{
    if (!c || !bvh || !orig || !dir || !maxt || !hits || nrays == 0 || nrays > c->cap)
        return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t mode_nostats = mode & ~RTA_TRACE_STATS;
    if (mode_nostats == RTA_TRACE_CIS) {
        // one launch traces every primary ray and, right after it, its bounce
        // ray; a gather then lays the bounce rays and hits out in primary order
        const uint32_t tiles = (nrays + kBounceTile - 1) / kBounceTile;
        RTA_CUDA_TRY(cudaMemsetAsync(c->tstat, 0, (size_t)tiles * 4, s));   // per-tile bounce counts
        RTA_CUDA_TRY(cudaMemsetAsync(&c->fs->queue, 0, 4, s));
        if (c->timing) RTA_CUDA_TRY(cudaEventRecord(c->ev_begin, s));
        int rc = trace_frame_fused(bvh, orig, dir, maxt, nrays, hits, seed, eps, c->s_orig, c->s_dir, c->s_hits,
                                   c->s_flag, c->tstat, &c->fs->queue, s);
        if (rc) return rc;
        if (c->timing) {
            RTA_CUDA_TRY(cudaEventRecord(c->ev_end, s));
            c->timed = true;
        }
        k_bounce_gather<<<tiles, kBounceThreads, 0, s>>>(c->s_flag, c->s_orig, c->s_dir, c->s_hits, nrays, c->orig,
                                                         c->dir, c->maxt, c->src, c->hits, c->tstat, c->fs);
        return check_launch("k_bounce_gather");
    }
    if (c->timing) RTA_CUDA_TRY(cudaEventRecord(c->ev_begin, s));
    const uint32_t rb = (nrays + 255) / 256 < 4096 ? (nrays + 255) / 256 : 4096;
    k_reset<<<rb, 256, 0, s>>>((HitRec *)hits, nrays, nullptr);
    int rc = check_launch("k_reset");
    if (rc) return rc;
    rc = trace_impl(bvh, orig, dir, maxt, nrays, nullptr, hits, mode_nostats, nullptr, &c->fs->queue, s);
    if (rc) return rc;
    rc = rta_diffuse_bounce(c, bvh, orig, dir, hits, nrays, seed, eps, stream);
    if (rc) return rc;
    k_reset<<<rb, 256, 0, s>>>(c->hits, nrays, &c->fs->count);
    if ((rc = check_launch("k_reset"))) return rc;
    rc = trace_impl(bvh, c->orig, c->dir, c->maxt, nrays, &c->fs->count, c->hits, mode_nostats, nullptr,
                    &c->fs->queue, s);
    if (rc) return rc;
    if (c->timing) {
        RTA_CUDA_TRY(cudaEventRecord(c->ev_end, s));
        c->timed = true;
    }
    return RTA_OK;
}

int rta_frame_set_timing(rta_frame_ctx *c, int on)
{
    if (!c) return RTA_ERR_INVALID;
    if (on && !c->ev_begin) {
        RTA_CUDA_TRY(cudaEventCreate(&c->ev_begin));
        RTA_CUDA_TRY(cudaEventCreate(&c->ev_end));
    }
    c->timing = on != 0;
    c->timed = false;
    return RTA_OK;
}

int rta_frame_trace_ms(rta_frame_ctx *c, float *ms)
{
    if (!c || !ms || !c->timed) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaEventSynchronize(c->ev_end));
    RTA_CUDA_TRY(cudaEventElapsedTime(ms, c->ev_begin, c->ev_end));
    return RTA_OK;
}

int rta_frame_status(rta_frame_ctx *c, rta_stream_t stream, uint32_t *flags)
{
    if (!c || !flags) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    FrameState fs;
    RTA_CUDA_TRY(cudaMemcpy(&fs, c->fs, sizeof(fs), cudaMemcpyDeviceToHost));
    *flags = fs.status;
    return RTA_OK;
}

} // extern "C"

// ------------------------------------------------------------------------- //
// allocation-free bounce                                                     //
// ------------------------------------------------------------------------- //
//
// Scratch of rta_diffuse_bounce_noalloc: 4 words of FrameState (tile counter,
// count, unused queue word, status flags) followed by one look-back word per
// 1024-ray tile, for at most RTA_BOUNCE_NOALLOC_MAX_RAYS rays: 64 KiB + 16 B.
// It is a module variable, so every GPU that loads the library holds it
// until the process exits, and every call shares it.

namespace rta {

static_assert(RTA_BOUNCE_NOALLOC_MAX_RAYS % kBounceTile == 0, "whole tiles");
constexpr uint32_t kNoAllocWords = 4u + RTA_BOUNCE_NOALLOC_MAX_RAYS / kBounceTile;
static __device__ __align__(256) uint32_t g_bounce_scratch[kNoAllocWords];

// host side: the device address of g_bounce_scratch, looked up once per
// device and context.  A context that was destroyed (cudaDeviceReset) and
// created again reloads the module, possibly at another address, so the
// cached address is keyed on the context's unique id (cuCtxGetId), which the
// driver never reuses.  The driver calls are fetched through the runtime, so
// the library does not link libcuda.
constexpr int kMaxDevices = 64;
static std::mutex g_scratch_mu;
static uint32_t *g_scratch_addr[kMaxDevices];
static unsigned long long g_scratch_ctx[kMaxDevices];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

static int current_context_id(int dev, unsigned long long *id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *f0 = nullptr, *f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
        RTA_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0));
        RTA_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1));
        if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1) {
            set_error_message("rta_diffuse_bounce_noalloc: the driver lacks cuCtxGetCurrent / cuCtxGetId");
            return RTA_ERR_CUDA;
        }
        get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS) {
        set_error_message("rta_diffuse_bounce_noalloc: cuCtxGetCurrent failed");
        return RTA_ERR_CUDA;
    }
    if (!ctx) {
        // no context bound to this thread yet: make the device's primary
        // context current (cudaSetDevice initialises it)
        RTA_CUDA_TRY(cudaSetDevice(dev));
        if (get_current(&ctx) != CUDA_SUCCESS || !ctx) {
            set_error_message("rta_diffuse_bounce_noalloc: no CUDA context");
            return RTA_ERR_CUDA;
        }
    }
    if (get_id(ctx, id) != CUDA_SUCCESS) {
        set_error_message("rta_diffuse_bounce_noalloc: cuCtxGetId failed");
        return RTA_ERR_CUDA;
    }
    return RTA_OK;
}

static int bounce_scratch(uint32_t **out)
{
    int dev = -1;
    RTA_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return RTA_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    unsigned long long ctx_id = 0;
    int rc = current_context_id(dev, &ctx_id);
    if (rc) return rc;
    if (!g_scratch_addr[dev] || g_scratch_ctx[dev] != ctx_id) {
        // The symbol's name is a host-side stand-in; only this call gives the
        // address the kernels of the current device may use.
        void *p = nullptr;
        RTA_CUDA_TRY(cudaGetSymbolAddress(&p, g_bounce_scratch));
        g_scratch_addr[dev] = static_cast<uint32_t *>(p);
        g_scratch_ctx[dev] = ctx_id;
    }
    *out = g_scratch_addr[dev];
    return RTA_OK;
}

} // namespace rta

static void g_bounce_noalloc_limit_error(uint32_t nrays)
{
    char msg[160];
    snprintf(msg, sizeof msg, "rta_diffuse_bounce_noalloc: %u rays exceed the %u-ray scratch", nrays,
             (unsigned)RTA_BOUNCE_NOALLOC_MAX_RAYS);
    rta::set_error_message(msg);
}

extern "C" int rta_diffuse_bounce_noalloc(const rta_lbvh *bvh, const float *orig, const float *dir,
                                          const void *hits, uint32_t nrays, uint32_t seed, float eps,
                                          float *out_orig, float *out_dir, float *out_maxt,
                                          uint32_t *out_src, uint32_t *out_count, uint32_t *out_flags,
                                          rta_stream_t stream)
{
    if (!bvh || !orig || !dir || !hits || !out_orig || !out_dir || !out_maxt || !out_src ||
        !out_count || nrays == 0)
        return RTA_ERR_INVALID;
    if (nrays > RTA_BOUNCE_NOALLOC_MAX_RAYS) {
        g_bounce_noalloc_limit_error(nrays);
        return RTA_ERR_INVALID;
    }
    uint32_t *scratch = nullptr;
    int rc = bounce_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t tiles = (nrays + kBounceTile - 1) / kBounceTile;
    // the tile counter, the count and the look-back words of this call start at zero
    RTA_CUDA_TRY(cudaMemsetAsync(scratch, 0, (size_t)(4u + tiles) * 4u, s));
    FrameState *fs = reinterpret_cast<FrameState *>(scratch);
    k_bounce<<<tiles, kBounceThreads, 0, s>>>((const TriRec *)bvh->tris, orig, dir, (const HitRec *)hits,
                                              nrays, seed, eps, out_orig, out_dir, out_maxt, out_src,
                                              scratch + 4, fs, bvh->n);
    if ((rc = check_launch("k_bounce (noalloc)"))) return rc;
    RTA_CUDA_TRY(cudaMemcpyAsync(out_count, &fs->count, 4, cudaMemcpyDeviceToDevice, s));
    // the call's device flags (a look-back wait that gave up leaves the
    // count and the ray order undefined); the next call clears the scratch
    if (out_flags) RTA_CUDA_TRY(cudaMemcpyAsync(out_flags, &fs->status, 4, cudaMemcpyDeviceToDevice, s));
    return RTA_OK;
}

// ------------------------------------------------------------------------- //
// host shading on the device: lighting_collector::reset / ::shade            //
// (librta/raytrav.h:186-233)                                                  //
// ------------------------------------------------------------------------- //
//
// One thread per pixel.  Lambert point lights with barycentric-interpolated
// vertex normals, in the reference's operation order (barycentric_coord in
// double, basic_types.h:90-94; barycentric_interpolation, tri.h:41-48;
// normalize_vec3f and dot_vec3f, cuda-vec.h:177-188) through round-to-nearest
// intrinsics, so the 8-bit image equals the host shader's byte for byte.

namespace rta {

constexpr uint32_t kMaxLights = 16;

struct ShadeLights {
    float l[kMaxLights][6];   // position xyz, colour rgb
    uint32_t n;
};

// int(x * 255) of the host shader (truncation; NaN -> 0, saturating)
__device__ __forceinline__ int to_int255(float x) { return __float2int_rz(__fmul_rn(x, 255.0f)); }

__device__ __forceinline__ float dot3_rn(const float *a, const float *b)
{
    float s = __fmul_rn(a[0], b[0]);
    s = __fadd_rn(s, __fmul_rn(a[1], b[1]));
    return __fadd_rn(s, __fmul_rn(a[2], b[2]));
}

__device__ __forceinline__ void normalize3_rn(float v[3])
{
    const float len = __fsqrt_rn(dot3_rn(v, v));
    v[0] = __fdiv_rn(v[0], len);
    v[1] = __fdiv_rn(v[1], len);
    v[2] = __fdiv_rn(v[2], len);
}

__device__ __forceinline__ void bary3_rn(float out[3], const float bc[3], const float *a, const float *b,
                                         const float *c)
{
#pragma unroll
    for (int k = 0; k < 3; ++k)
        out[k] = __fadd_rn(__fadd_rn(__fmul_rn(a[k], bc[0]), __fmul_rn(b[k], bc[1])), __fmul_rn(c[k], bc[2]));
}

__global__ void k_shade_reset(uint8_t *__restrict__ img, uint32_t n, uchar3 bg)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        img[3 * (size_t)i + 0] = bg.x;
        img[3 * (size_t)i + 1] = bg.y;
        img[3 * (size_t)i + 2] = bg.z;
    }
}

__global__ void k_shade_lambert(const HitRec *__restrict__ hits, const float *__restrict__ tris, uint32_t n_tris,
                                uint32_t n, ShadeLights L, int binary, uint8_t *__restrict__ img,
                                uint32_t *__restrict__ flags)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const HitRec is = hits[i];
        if (is.t == FLT_MAX) continue;
        float col[3] = {0.0f, 0.0f, 0.0f};
        if (binary) {
            col[0] = L.l[0][3];
            col[1] = L.l[0][4];
            col[2] = L.l[0][5];
        } else {
            if (is.ref >= n_tris) {
                if (flags) atomicOr(flags, RTA_DEV_BAD_LINK);
                continue;
            }
            const float *t = tris + (size_t)is.ref * 26;
            float va[9], na[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                va[k] = __ldg(t + k);
                na[k] = __ldg(t + 9 + k);
            }
            // x = 1.0 - beta - gamma, evaluated in double and stored as float
            const float bc[3] = {__double2float_rn(__dsub_rn(__dsub_rn(1.0, (double)is.beta), (double)is.gamma)),
                                 is.beta, is.gamma};
            for (uint32_t l = 0; l < L.n; ++l) {
                float N[3], p[3];
                bary3_rn(N, bc, na, na + 3, na + 6);
                bary3_rn(p, bc, va, va + 3, va + 6);
                float D[3] = {__fsub_rn(L.l[l][0], p[0]), __fsub_rn(L.l[l][1], p[1]), __fsub_rn(L.l[l][2], p[2])};
                normalize3_rn(D);
                normalize3_rn(N);
                float d = dot3_rn(N, D);
                d = (d < 0.0f) ? 0.0f : d;   // std::max(dot, 0)
#pragma unroll
                for (int k = 0; k < 3; ++k) col[k] = __fadd_rn(col[k], __fmul_rn(L.l[l][3 + k], d));
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            int v = to_int255(col[k]);
            v = v < 255 ? v : 255;
            img[3 * (size_t)i + k] = (uint8_t)(v > 0 ? v : 0);
        }
    }
}

} // namespace rta

extern "C" int rta_shade_lambert(const void *hits, const void *tris, uint32_t n_tris, uint32_t w, uint32_t h,
                                 const float *lights, uint32_t n_lights, int binary_only, const float *background,
                                 void *image, uint32_t *d_flags, rta_stream_t stream)
{
    if (!hits || !image || w == 0 || h == 0 || n_lights > kMaxLights || (n_lights && !lights) ||
        (n_lights && !binary_only && (!tris || n_tris == 0)) || (uint64_t)w * h > 0xffffffffull)
        return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t n = w * h;
    const uint32_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    if (background) {
        // reset (raytrav.h:189-194): min(int(c * 255), 255) stored as a byte
        unsigned char b[3];
        for (int k = 0; k < 3; ++k) {
            const float v = background[k] * 255.0f;
            long iv = (v != v) ? 0 : (v >= 2147483647.0f ? 2147483647L : (v <= -2147483648.0f ? -2147483648L : (long)v));
            b[k] = (unsigned char)(iv < 255 ? iv : 255);
        }
        k_shade_reset<<<blocks, 256, 0, s>>>((uint8_t *)image, n, make_uchar3(b[0], b[1], b[2]));
        int rc = check_launch("k_shade_reset");
        if (rc) return rc;
    }
    if (n_lights == 0) return RTA_OK;   // shade() returns at once without lights
    ShadeLights L;
    memset(&L, 0, sizeof(L));
    memcpy(L.l, lights, (size_t)n_lights * 6 * sizeof(float));
    L.n = n_lights;
    k_shade_lambert<<<blocks, 256, 0, s>>>((const HitRec *)hits, (const float *)tris, n_tris, n, L, binary_only,
                                           (uint8_t *)image, d_flags);
    return check_launch("k_shade_lambert");
}

// ------------------------------------------------------------------------- //
// frames on host buffers, pipelined                                          //
// ------------------------------------------------------------------------- //
//
// A renderer that keeps its rays and hits in host memory calls one frame
// after another.  Each call copies its rays in on one stream, traces the
// frame (rta_frame_run) on a second, and copies its hits out on a third,
// with two sets of device buffers used in turn, so that the copies of one
// frame overlap the traversal of its neighbours:
//
//   h2d    H2D rays(k)                       H2D rays(k+1)
//   comp                 frame(k)                            frame(k+1)
//   d2h                            D2H hits(k)                          ...
//
// Events order the three streams: frame k waits for its rays; the rays of
// frame k+2 (same buffers as k) wait until frame k's hits are out.

namespace rta {

} // namespace rta

struct rta_host_frames {
    uint32_t cap = 0;
    rta_frame_ctx *slot[2] = {nullptr, nullptr};
    float *orig[2] = {nullptr, nullptr}, *dir[2] = {nullptr, nullptr}, *maxt[2] = {nullptr, nullptr};
    HitRec *hits[2] = {nullptr, nullptr};
    cudaStream_t h2d = nullptr, comp = nullptr, d2h = nullptr;
    cudaEvent_t in_done[2] = {nullptr, nullptr}, comp_done[2] = {nullptr, nullptr}, out_done[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    uint32_t next = 0;
};

static void free_host_frames(rta_host_frames *p)
{
    for (int k = 0; k < 2; ++k) {
        if (p->slot[k]) rta_frame_destroy(p->slot[k]);
        void *ptrs[] = {p->orig[k], p->dir[k], p->maxt[k], p->hits[k]};
        for (void *q : ptrs)
            if (q) cudaFree(q);
        cudaEvent_t evs[] = {p->in_done[k], p->comp_done[k], p->out_done[k]};
        for (cudaEvent_t e : evs)
            if (e) cudaEventDestroy(e);
    }
    cudaStream_t ss[] = {p->h2d, p->comp, p->d2h};
    for (cudaStream_t s : ss)
        if (s) cudaStreamDestroy(s);
}

extern "C" {

int rta_host_frames_create(rta_host_frames **out, uint32_t max_rays)
{
    if (!out || max_rays == 0) return RTA_ERR_INVALID;
    rta_host_frames *p = new rta_host_frames();
    p->cap = max_rays;
    auto fail = [&](int rc) {
        free_host_frames(p);
        delete p;
        return rc;
    };
    int rc;
    for (int k = 0; k < 2; ++k) {
        if ((rc = rta_frame_create(&p->slot[k], max_rays))) return fail(rc);
        cudaError_t e = cudaSuccess;
        if (e == cudaSuccess) e = cudaMalloc(&p->orig[k], (size_t)max_rays * 12);
        if (e == cudaSuccess) e = cudaMalloc(&p->dir[k], (size_t)max_rays * 12);
        if (e == cudaSuccess) e = cudaMalloc(&p->maxt[k], (size_t)max_rays * 4);
        if (e == cudaSuccess) e = cudaMalloc(&p->hits[k], (size_t)max_rays * sizeof(HitRec));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->in_done[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->comp_done[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->out_done[k], cudaEventDisableTiming);
        if (e != cudaSuccess) {
            set_cuda_error(e, "rta_host_frames_create");
            return fail(e == cudaErrorMemoryAllocation ? RTA_ERR_NOMEM : RTA_ERR_CUDA);
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&p->h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->d2h, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_cuda_error(e, "rta_host_frames_create");
        return fail(RTA_ERR_CUDA);
    }
    *out = p;
    return RTA_OK;
}

int rta_host_frames_destroy(rta_host_frames *p)
{
    if (!p) return RTA_ERR_INVALID;
    cudaStreamSynchronize(p->h2d);
    cudaStreamSynchronize(p->comp);
    cudaStreamSynchronize(p->d2h);
    free_host_frames(p);
    delete p;
    return RTA_OK;
}

int rta_host_frames_run(rta_host_frames *p, const rta_lbvh *bvh, const float *h_orig, const float *h_dir,
                        const float *h_maxt, uint32_t nrays, void *h_hits, void *h_bounce_hits,
                        uint32_t *h_bounce_count, uint32_t mode, uint32_t seed, float eps, rta_stream_t stream)
{
    if (!p || !bvh || !h_orig || !h_dir || !h_maxt || !h_hits || !h_bounce_hits || !h_bounce_count || nrays == 0 ||
        nrays > p->cap)
        return RTA_ERR_INVALID;
    const uint32_t k = p->next;
    p->next ^= 1u;
    rta_frame_ctx *f = p->slot[k];
    // rays in, once frame k-2's hits (same buffers) are out
    if (p->used[k]) RTA_CUDA_TRY(cudaStreamWaitEvent(p->h2d, p->out_done[k], 0));
    RTA_CUDA_TRY(cudaMemcpyAsync(p->orig[k], h_orig, (size_t)nrays * 12, cudaMemcpyHostToDevice, p->h2d));
    RTA_CUDA_TRY(cudaMemcpyAsync(p->dir[k], h_dir, (size_t)nrays * 12, cudaMemcpyHostToDevice, p->h2d));
    RTA_CUDA_TRY(cudaMemcpyAsync(p->maxt[k], h_maxt, (size_t)nrays * 4, cudaMemcpyHostToDevice, p->h2d));
    RTA_CUDA_TRY(cudaEventRecord(p->in_done[k], p->h2d));
    // the frame, once its rays are in and the tree's last build (on whatever
    // stream it was issued) is complete
    RTA_CUDA_TRY(cudaStreamWaitEvent(p->comp, p->in_done[k], 0));
    if (bvh->ready) RTA_CUDA_TRY(cudaStreamWaitEvent(p->comp, (cudaEvent_t)bvh->ready, 0));
    int rc = rta_frame_run(f, bvh, p->orig[k], p->dir[k], p->maxt[k], nrays, p->hits[k], mode, seed, eps, p->comp);
    if (rc) return rc;
    RTA_CUDA_TRY(cudaEventRecord(p->comp_done[k], p->comp));
    // hits out
    RTA_CUDA_TRY(cudaStreamWaitEvent(p->d2h, p->comp_done[k], 0));
    RTA_CUDA_TRY(cudaMemcpyAsync(h_hits, p->hits[k], (size_t)nrays * sizeof(HitRec), cudaMemcpyDeviceToHost, p->d2h));
    RTA_CUDA_TRY(cudaMemcpyAsync(h_bounce_count, &f->fs->count, 4, cudaMemcpyDeviceToHost, p->d2h));
    // all nrays bounce slots (the count is known only on the device): a copy
    // engine moves them beside the next frame's traversal, where a copy
    // kernel of exactly `count` records would wait for that frame's blocks
    RTA_CUDA_TRY(cudaMemcpyAsync(h_bounce_hits, f->hits, (size_t)nrays * sizeof(HitRec), cudaMemcpyDeviceToHost,
                                 p->d2h));
    RTA_CUDA_TRY(cudaEventRecord(p->out_done[k], p->d2h));
    p->used[k] = true;
    // the caller's stream sees this frame's results once it passes here
    RTA_CUDA_TRY(cudaStreamWaitEvent((cudaStream_t)stream, p->out_done[k], 0));
    return RTA_OK;
}

} // extern "C"
