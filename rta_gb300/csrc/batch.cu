// batch.cu -- batched multi-mesh LBVH build and trace on sm_103a.
//
// M independent meshes are built in one pass sequence over the concatenated
// triangles instead of M one-mesh builds:
//   init     per-mesh boxes to the reference's +-1e11 start values
//   bounds   centroids; per-mesh boxes by warp-segmented min/max of
//            order-preserving integer keys and one atomic per warp and mesh
//   morton   per-mesh d = GRID / extent, 30-bit code, key = mesh << 30 | code,
//            digit histograms of every sort pass
//   sort     onesweep LSD passes over the (mesh, code) keys; the last pass
//            also writes each key's 30-bit code for the trees
//   karras   every inner node of every mesh (its mesh is the key's top bits),
//            Morton-ordered triangles, mesh-local ids
//   refit    the range refit of lbvh.cuh over all meshes' leaves at once
//            (a node's range never leaves its mesh; each mesh's root record
//            takes its root's box)
// and traced by one persistent launch over all rays (k_trace_batch in
// trace.cu).  Because a stable sort by (mesh, code) orders each mesh's
// triangles exactly as a sort by code alone does, and every per-mesh step
// runs the one-mesh code (lbvh.cuh) on the mesh's own ranges, every mesh's
// tree equals its one-mesh build bit for bit.  rta_batch_run replays the
// whole sequence (plus the hit reset and the trace) as one CUDA graph.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "batch.cuh"
#include "lbvh.cuh"

namespace rta {

constexpr uint32_t kMaxMeshes = 1u << 20;
constexpr uint32_t kCodeMask30 = (1u << 30) - 1u;

// per-mesh scene box as order-preserving integer keys (min/max of the keys =
// min/max of the floats; -0 orders below +0, which changes no code)
struct BoxKeys {
    uint32_t lo[3], hi[3], pad[2];
};

__device__ __forceinline__ uint32_t f2o(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float o2f(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void k_batch_init(BoxKeys *__restrict__ box, uint32_t meshes)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= meshes) return;
    // calculateVoxelBounds starts from +-1e11 (lbvh-kernels.cu:519-520)
    BoxKeys b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = f2o(100000000000.0f);
        b.hi[k] = f2o(-100000000000.0f);
    }
    b.pad[0] = b.pad[1] = 0;
    box[m] = b;
}

// centroids and per-mesh boxes
__global__ void __launch_bounds__(256)
k_batch_bounds(const float *__restrict__ tris, uint32_t n, const uint32_t *__restrict__ tri_off,
               uint32_t meshes, float *__restrict__ cent, BoxKeys *__restrict__ box)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp * 32u; base < n; base += warps * 32u) {
        const uint32_t i = base + lane;
        const bool ok = i < n;
        uint32_t m = 0xffffffffu;
        uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
        if (ok) {
            m = find_range(tri_off, meshes, i);
            float a[3], b[3], c[3];
            load_positions(tris + (size_t)i * kTriFloats, a, b, c);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                // aabbOfTri (:141-153); centroid ((a+b)+c)/3.0f (:60-63)
                lo[k] = f2o(ref_min(ref_min(a[k], b[k]), c[k]));
                hi[k] = f2o(ref_max(ref_max(a[k], b[k]), c[k]));
                cent[(size_t)i * 3 + k] = __fdiv_rn(__fadd_rn(__fadd_rn(a[k], b[k]), c[k]), 3.0f);
            }
        }
        // lanes of one mesh are contiguous; each group reduces and its first
        // lane folds the group's box into the mesh's
        const uint32_t group = __match_any_sync(0xffffffffu, m);
        uint32_t rlo[3], rhi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            rlo[k] = __reduce_min_sync(group, lo[k]);
            rhi[k] = __reduce_max_sync(group, hi[k]);
        }
        if (ok && (int)lane == __ffs(group) - 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                atomicMin(&box[m].lo[k], rlo[k]);
                atomicMax(&box[m].hi[k], rhi[k]);
            }
        }
    }
}

// keys = mesh << 30 | 30-bit code over the mesh's box, and the digit
// histograms of every sort pass
template <int DBITS>
__global__ void __launch_bounds__(256)
k_batch_morton(const float *__restrict__ cent, uint32_t n, const uint32_t *__restrict__ tri_off,
               uint32_t meshes, const BoxKeys *__restrict__ box, uint64_t *__restrict__ keys,
               SortScratchHeader *__restrict__ hdr, uint32_t *__restrict__ flags, int passes)
{
    extern __shared__ uint32_t s_hist[];
    constexpr int radix = 1 << DBITS;
    for (int j = threadIdx.x; j < passes * radix; j += blockDim.x) s_hist[j] = 0;
    __syncthreads();
    bool wrapped = false, flat = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t m = find_range(tri_off, meshes, i);
        const BoxKeys bk = box[m];
        float lo[3], d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = o2f(bk.lo[k]);
            // d = GRIDSIZE / (max - min), on the host in the reference (:414-417)
            d[k] = __fdiv_rn(1024.0f, __fsub_rn(o2f(bk.hi[k]), lo[k]));
            flat |= !isfinite(d[k]);
        }
        const float c[3] = {cent[(size_t)i * 3 + 0], cent[(size_t)i * 3 + 1], cent[(size_t)i * 3 + 2]};
        const uint64_t key = ((uint64_t)m << 30) | morton_code(c, lo, d, 0x3ffu, wrapped);
        keys[i] = key;
        hist_add<DBITS>(s_hist, key, passes);
    }
    if (__any_sync(0xffffffffu, wrapped) && (threadIdx.x & 31) == 0) atomicOr(flags, RTA_DEV_QUANT_WRAP);
    if (__any_sync(0xffffffffu, flat) && (threadIdx.x & 31) == 0) atomicOr(flags, RTA_DEV_ZERO_EXTENT);
    __syncthreads();
    for (int j = threadIdx.x; j < passes * radix; j += blockDim.x)
        if (s_hist[j]) atomicAdd(hdr->hist + j, s_hist[j]);
}

// every inner node of every mesh; with tris, also the Morton-ordered
// triangles and the mesh-local ids (else the refit's, k_refit_seg)
__global__ void __launch_bounds__(256)
k_batch_karras(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ codes, uint32_t n,
               const MeshRec *__restrict__ meshes, uint4 *__restrict__ links, uint32_t *__restrict__ parents,
               const float *__restrict__ tris_in, uint32_t *__restrict__ ids, TriRec *__restrict__ tris)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const MeshRec mr = meshes[(uint32_t)(keys[i] >> 30)];
    const uint32_t li = i - mr.tri_off;
    TriRec tr;
    uint32_t lid = 0;
    if (tris) {
        const uint32_t id = __ldg(ids + i);
        lid = id - mr.tri_off;
        tr = make_tri(tris_in + (size_t)id * kTriFloats, lid);
    }
    if (li + 1 < mr.n_tris)
        karras_node(codes + mr.tri_off, mr.n_tris, li, links + mr.node_off, parents + mr.parent_off, mr.tri_off);
    if (tris) {
        tris[i] = tr;
        ids[i] = lid;
    }
}

// reset_intersections (librta/cuda-kernels.cu:24-44): t, beta, gamma; ref kept
__global__ void k_batch_reset_hits(HitRec *__restrict__ hits, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        hits[i].t = FLT_MAX;
        hits[i].beta = 1.0f;
        hits[i].gamma = 2.0f;
    }
}

static int batch_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

static bool valid_params(const rta_batch_params &p)
{
    return (p.digit_bits >= 8 && p.digit_bits <= 11) && p.fetch_idle >= 1 &&
           p.fetch_idle <= 32 && p.blocks_per_sm >= 0 && p.blocks_per_sm <= 64 && (p.stack == 40 || p.stack == 64);
}

} // namespace rta

using namespace rta;

struct rta_batch {
    // meshes
    uint32_t meshes = 0, n = 0, rays = 0, mesh_bits = 0;
    std::vector<uint32_t> h_tri_off, h_ray_off;
    std::vector<MeshRec> h_meshes;
    rta_batch_params params = {8, 12, 0, 40};
    // device buffers
    MeshRec *meshes_d = nullptr;
    uint32_t *tri_off_d = nullptr, *ray_off_d = nullptr;
    BoxKeys *box = nullptr;
    float *cent = nullptr;
    uint64_t *keys0 = nullptr, *keys1 = nullptr;
    uint32_t *vals0 = nullptr, *vals1 = nullptr;
    uint32_t *codes = nullptr;
    unsigned char *scratch = nullptr;   // SortScratchHeader + tile status words
    NodeRec *nodes = nullptr;
    RootRec *roots = nullptr;
    uint32_t *parents = nullptr, *counters = nullptr;   // counters: the refit's crossing-node list
    uint4 *links = nullptr;                              // Karras links per inner node, read by the refit
    TriRec *tris = nullptr;
    uint32_t *status = nullptr;         // [0] flags, [4] trace queue
    float *rbox = nullptr;              // refit tables (refit_layout)
    // result of the last build
    const uint64_t *keys_sorted = nullptr;
    uint32_t *index = nullptr;
    bool built = false;
    // graph of rta_batch_run
    cudaGraphExec_t exec = nullptr;
    const void *g_tris = nullptr;
    const float *g_orig = nullptr, *g_dir = nullptr, *g_maxt = nullptr;
    void *g_hits = nullptr;
    rta_batch_params g_params = {0, 0, 0, 0};
};

static void free_batch(rta_batch *b)
{
    void *ptrs[] = {b->meshes_d, b->tri_off_d, b->ray_off_d, b->box, b->cent, b->keys0, b->keys1,
                    b->vals0, b->vals1, b->codes, b->scratch, b->nodes, b->roots, b->parents,
                    b->counters, b->tris, b->status, b->rbox, b->links};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    const rta_batch_params keep = b->params;
    *b = rta_batch();
    b->params = keep;
}

// tile status words per tile: the most any supported digit width needs
static size_t batch_status_words(int key_bits)
{
    size_t w = 0;
    for (int d : {8, 9, 10, 11}) w = std::max(w, (size_t)sort_passes(key_bits, d) << d);
    return w;
}

static int batch_build_impl(rta_batch *b, const void *tris, cudaStream_t s)
{
    const uint32_t n = b->n;
    const int db = b->params.digit_bits;
    const int key_bits = 30 + (int)b->mesh_bits;
    const int passes = sort_passes(key_bits, db);
    if (passes > kMaxPasses) {
        set_error_message("rta_batch_build: too many sort passes for this digit width");
        return RTA_ERR_INVALID;
    }
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    SortScratchHeader *hdr = reinterpret_cast<SortScratchHeader *>(b->scratch);
    uint32_t *tstat = reinterpret_cast<uint32_t *>(b->scratch + sizeof(SortScratchHeader));
    RTA_CUDA_TRY(cudaMemsetAsync(b->scratch, 0, sizeof(SortScratchHeader) + ((size_t)passes << db) * tiles * 4, s));
    RTA_CUDA_TRY(cudaMemsetAsync(b->status, 0, 4, s));
    k_batch_init<<<(b->meshes + 255) / 256, 256, 0, s>>>(b->box, b->meshes);
    int rc = check_launch("k_batch_init");
    if (rc) return rc;
    const float *tin = static_cast<const float *>(tris);
    const uint32_t eb = (n + 255) / 256;
    const uint32_t grid = std::min<uint32_t>(eb, (uint32_t)batch_sms() * 8u);
    k_batch_bounds<<<grid, 256, 0, s>>>(tin, n, b->tri_off_d, b->meshes, b->cent, b->box);
    if ((rc = check_launch("k_batch_bounds"))) return rc;
    {
        const size_t hs = ((size_t)passes << db) * 4;
        switch (db) {
        case 9:
            k_batch_morton<9><<<grid, 256, hs, s>>>(b->cent, n, b->tri_off_d, b->meshes, b->box, b->keys0, hdr,
                                                    b->status, passes);
            break;
        case 10:
            k_batch_morton<10><<<grid, 256, hs, s>>>(b->cent, n, b->tri_off_d, b->meshes, b->box, b->keys0, hdr,
                                                     b->status, passes);
            break;
        case 11:
            k_batch_morton<11><<<grid, 256, hs, s>>>(b->cent, n, b->tri_off_d, b->meshes, b->box, b->keys0, hdr,
                                                     b->status, passes);
            break;
        default:
            k_batch_morton<8><<<grid, 256, hs, s>>>(b->cent, n, b->tri_off_d, b->meshes, b->box, b->keys0, hdr,
                                                    b->status, passes);
        }
    }
    if ((rc = check_launch("k_batch_morton"))) return rc;
    uint64_t *ks = nullptr;
    uint32_t *vs = nullptr;
    switch (db) {
    case 9:
        rc = sort_passes_launch<uint64_t, 9>(b->keys0, b->keys1, b->vals0, b->vals1, n, passes, hdr, tstat,
                                             b->status, b->codes, kCodeMask30, s, &ks, &vs);
        break;
    case 10:
        rc = sort_passes_launch<uint64_t, 10>(b->keys0, b->keys1, b->vals0, b->vals1, n, passes, hdr, tstat,
                                              b->status, b->codes, kCodeMask30, s, &ks, &vs);
        break;
    case 11:
        rc = sort_passes_launch<uint64_t, 11>(b->keys0, b->keys1, b->vals0, b->vals1, n, passes, hdr, tstat,
                                              b->status, b->codes, kCodeMask30, s, &ks, &vs);
        break;
    default:
        rc = sort_passes_launch<uint64_t, 8>(b->keys0, b->keys1, b->vals0, b->vals1, n, passes, hdr, tstat,
                                             b->status, b->codes, kCodeMask30, s, &ks, &vs);
    }
    if (rc) return rc;
    b->keys_sorted = ks;
    b->index = vs;
    TriRec *kg = RTA_KARRAS_GATHER ? b->tris : nullptr;
    k_batch_karras<<<eb, 256, 0, s>>>(ks, b->codes, n, b->meshes_d, b->links, b->parents, tin, vs, kg);
    if ((rc = check_launch("k_batch_karras"))) return rc;
    const uint32_t inner = n - b->meshes;
    rc = refit_launch<uint32_t, true>(b->codes, n, b->meshes_d, ks, kg ? nullptr : tin, vs, b->nodes, b->links, b->parents, b->tris,
                                      b->roots, b->rbox, b->counters, inner ? inner : 1u, &hdr->n_cross, &hdr->refit_ticket,
                                      b->status, batch_sms(), s);
    if (rc) return rc;
    b->built = true;
    return RTA_OK;
}

static int batch_trace_impl(rta_batch *b, const float *orig, const float *dir, const float *maxt, void *hits,
                            uint32_t *stats, cudaStream_t s)
{
    if (b->rays == 0) return RTA_OK;
    BatchTraceArgs a;
    a.nodes = b->nodes;
    a.roots = b->roots;
    a.tris = b->tris;
    a.meshes = b->meshes_d;
    a.ray_off = b->ray_off_d;
    a.n_meshes = b->meshes;
    a.orig = orig;
    a.dir = dir;
    a.maxt = maxt;
    a.nrays = b->rays;
    a.hits = (HitRec *)hits;
    a.stats = stats;
    a.queue = b->status + 4;
    a.status = b->status;
    a.fetch_idle = b->params.fetch_idle;
    RTA_CUDA_TRY(cudaMemsetAsync(a.queue, 0, 4, s));
    return launch_batch_trace(a, b->params.stack, b->params.blocks_per_sm, s);
}

// everything a graph capture must not do itself: kernel attributes and
// occupancy queries of every kernel the batch launches
static int batch_prepare(rta_batch *b)
{
    static bool done = false;
    if (done) return RTA_OK;
    RTA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint64_t, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(SortSmem<uint64_t, 8>)));
    RTA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint64_t, 10>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(SortSmem<uint64_t, 10>)));
    RTA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint64_t, 11>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(SortSmem<uint64_t, 11>)));
    batch_trace_max_blocks_per_sm(40);
    batch_trace_max_blocks_per_sm(64);
    batch_sms();
    (void)b;
    done = true;
    return RTA_OK;
}


extern "C" {

int rta_batch_create(rta_batch **out)
{
    if (!out) return RTA_ERR_INVALID;
    *out = new rta_batch();
    return RTA_OK;
}

int rta_batch_destroy(rta_batch *b)
{
    if (!b) return RTA_ERR_INVALID;
    free_batch(b);
    delete b;
    return RTA_OK;
}

int rta_batch_set_meshes(rta_batch *b, uint32_t meshes, const uint32_t *tri_offsets,
                         const uint32_t *ray_offsets)
{
    if (!b || meshes == 0 || meshes > kMaxMeshes || !tri_offsets || !ray_offsets) return RTA_ERR_INVALID;
    if (tri_offsets[0] != 0 || ray_offsets[0] != 0) return RTA_ERR_INVALID;
    std::vector<MeshRec> mr(meshes);
    for (uint32_t m = 0; m < meshes; ++m) {
        if (tri_offsets[m + 1] <= tri_offsets[m] || ray_offsets[m + 1] < ray_offsets[m]) return RTA_ERR_INVALID;
        const uint32_t nt = tri_offsets[m + 1] - tri_offsets[m];
        if (nt > kMaxTriangles) return RTA_ERR_INVALID;
        mr[m].tri_off = tri_offsets[m];
        mr[m].n_tris = nt;
        mr[m].node_off = tri_offsets[m] - m;
        mr[m].parent_off = 2u * tri_offsets[m] - m;
        mr[m].ray_off = ray_offsets[m];
        mr[m].n_rays = ray_offsets[m + 1] - ray_offsets[m];
        mr[m].pad0 = mr[m].pad1 = 0;
    }
    const uint64_t n = tri_offsets[meshes];
    if (n > 0xffffffffull / 2) return RTA_ERR_INVALID;
    free_batch(b);
    b->meshes = meshes;
    b->n = (uint32_t)n;
    b->rays = ray_offsets[meshes];
    b->mesh_bits = 0;
    while ((1u << b->mesh_bits) < meshes) ++b->mesh_bits;
    b->h_tri_off.assign(tri_offsets, tri_offsets + meshes + 1);
    b->h_ray_off.assign(ray_offsets, ray_offsets + meshes + 1);
    b->h_meshes = mr;
    const uint32_t nn = b->n;
    const uint32_t tiles = (nn + kSortTile - 1) / kSortTile;
    RTA_CUDA_TRY(cudaMalloc(&b->meshes_d, (size_t)meshes * sizeof(MeshRec)));
    RTA_CUDA_TRY(cudaMalloc(&b->tri_off_d, (size_t)(meshes + 1) * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->ray_off_d, (size_t)(meshes + 1) * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->box, (size_t)meshes * sizeof(BoxKeys)));
    RTA_CUDA_TRY(cudaMalloc(&b->cent, (size_t)nn * 12));
    RTA_CUDA_TRY(cudaMalloc(&b->keys0, (size_t)nn * 8));
    RTA_CUDA_TRY(cudaMalloc(&b->keys1, (size_t)nn * 8));
    RTA_CUDA_TRY(cudaMalloc(&b->vals0, (size_t)nn * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->vals1, (size_t)nn * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->codes, (size_t)nn * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->scratch, sizeof(SortScratchHeader) +
                                             batch_status_words(30 + (int)b->mesh_bits) * tiles * 4));
    const size_t inner = nn - meshes;
    RTA_CUDA_TRY(cudaMalloc(&b->nodes, (inner ? inner : 1) * sizeof(NodeRec)));
    RTA_CUDA_TRY(cudaMalloc(&b->roots, (size_t)meshes * sizeof(RootRec)));
    RTA_CUDA_TRY(cudaMalloc(&b->parents, (2 * (size_t)nn - meshes) * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->counters, (inner ? inner : 1) * 4));
    RTA_CUDA_TRY(cudaMalloc(&b->links, (inner ? inner : 1) * sizeof(uint4)));
    RTA_CUDA_TRY(cudaMalloc(&b->rbox, refit_layout(nn).total * 6 * sizeof(float)));
    RTA_CUDA_TRY(cudaMalloc(&b->tris, (size_t)nn * sizeof(TriRec)));
    RTA_CUDA_TRY(cudaMalloc(&b->status, 64));
    RTA_CUDA_TRY(cudaMemset(b->status, 0, 64));
    RTA_CUDA_TRY(cudaMemcpy(b->meshes_d, mr.data(), (size_t)meshes * sizeof(MeshRec), cudaMemcpyHostToDevice));
    RTA_CUDA_TRY(cudaMemcpy(b->tri_off_d, tri_offsets, (size_t)(meshes + 1) * 4, cudaMemcpyHostToDevice));
    RTA_CUDA_TRY(cudaMemcpy(b->ray_off_d, ray_offsets, (size_t)(meshes + 1) * 4, cudaMemcpyHostToDevice));
    return RTA_OK;
}

int rta_batch_build(rta_batch *b, const void *tris, rta_stream_t stream)
{
    if (!b || !tris || b->meshes == 0) return RTA_ERR_INVALID;
    int rc = batch_prepare(b);
    if (rc) return rc;
    return batch_build_impl(b, tris, (cudaStream_t)stream);
}

int rta_batch_trace(rta_batch *b, const float *orig, const float *dir, const float *maxt, void *hits,
                    uint32_t *stats, rta_stream_t stream)
{
    if (!b || !b->built || (b->rays && (!orig || !dir || !maxt || !hits))) return RTA_ERR_INVALID;
    int rc = batch_prepare(b);
    if (rc) return rc;
    return batch_trace_impl(b, orig, dir, maxt, hits, stats, (cudaStream_t)stream);
}

int rta_batch_run(rta_batch *b, const void *tris, const float *orig, const float *dir, const float *maxt,
                  void *hits, rta_stream_t stream)
{
    if (!b || !tris || b->meshes == 0 || (b->rays && (!orig || !dir || !maxt || !hits))) return RTA_ERR_INVALID;
    int rc = batch_prepare(b);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const rta_batch_params &p = b->params;
    const bool same = b->exec && b->g_tris == tris && b->g_orig == orig && b->g_dir == dir &&
                      b->g_maxt == maxt && b->g_hits == hits && b->g_params.digit_bits == p.digit_bits &&
                      b->g_params.fetch_idle == p.fetch_idle && b->g_params.blocks_per_sm == p.blocks_per_sm &&
                      b->g_params.stack == p.stack;
    if (!same) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        // the capturing stream must not be the legacy default stream
        cudaStream_t cs = s;
        cudaStream_t own = nullptr;
        if (s == nullptr || s == cudaStreamLegacy) {
            RTA_CUDA_TRY(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
            cs = own;
        }
        cudaGraph_t g = nullptr;
        RTA_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
        rc = batch_build_impl(b, tris, cs);
        if (!rc && b->rays) {
            k_batch_reset_hits<<<std::min<uint32_t>((b->rays + 255) / 256, (uint32_t)batch_sms() * 8u), 256, 0,
                                 cs>>>((HitRec *)hits, b->rays);
            rc = check_launch("k_batch_reset_hits");
            if (!rc) rc = batch_trace_impl(b, orig, dir, maxt, hits, nullptr, cs);
        }
        cudaError_t e = cudaStreamEndCapture(cs, &g);
        if (!rc && e != cudaSuccess) {
            set_cuda_error(e, "cudaStreamEndCapture");
            rc = RTA_ERR_CUDA;
        }
        if (!rc) {
            e = cudaGraphInstantiate(&b->exec, g, 0);
            if (e != cudaSuccess) {
                set_cuda_error(e, "cudaGraphInstantiate");
                rc = RTA_ERR_CUDA;
                b->exec = nullptr;
            }
        }
        if (g) cudaGraphDestroy(g);
        if (own) cudaStreamDestroy(own);
        if (rc) return rc;
        b->g_tris = tris;
        b->g_orig = orig;
        b->g_dir = dir;
        b->g_maxt = maxt;
        b->g_hits = hits;
        b->g_params = p;
    }
    RTA_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    return RTA_OK;
}

int rta_batch_mesh(const rta_batch *b, uint32_t mesh, rta_lbvh *out)
{
    if (!b || !out || !b->built || mesh >= b->meshes) return RTA_ERR_INVALID;
    const MeshRec &mr = b->h_meshes[mesh];
    out->nodes = b->nodes + mr.node_off;
    out->root = b->roots + mesh;
    out->tris = b->tris + mr.tri_off;
    out->index = b->index + mr.tri_off;
    out->codes = b->codes + mr.tri_off;
    out->parents = b->parents + mr.parent_off;
    out->n = mr.n_tris;
    out->morton_bits = 30;
    out->status = b->status;
    out->ready = nullptr;   // the caller orders the batch build before other streams' use
    return RTA_OK;
}

int rta_batch_status(const rta_batch *b, rta_stream_t stream, uint32_t *flags)
{
    if (!b || !flags || !b->status) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    RTA_CUDA_TRY(cudaMemcpy(flags, b->status, 4, cudaMemcpyDeviceToHost));
    return RTA_OK;
}

int rta_batch_get_params(const rta_batch *b, rta_batch_params *p)
{
    if (!b || !p) return RTA_ERR_INVALID;
    *p = b->params;
    return RTA_OK;
}

int rta_batch_set_params(rta_batch *b, const rta_batch_params *p)
{
    if (!b || !p || !valid_params(*p)) return RTA_ERR_INVALID;
    if (b->meshes && sort_passes(30 + (int)b->mesh_bits, p->digit_bits) > kMaxPasses) return RTA_ERR_INVALID;
    b->params = *p;
    return RTA_OK;
}

} // extern "C"

// ------------------------------------------------------------------------- //
// autotuner and its cache                                                    //
// ------------------------------------------------------------------------- //
//
// The cache is a JSON object with one entry per line:
//   "key": {"digit_bits": 8, "fetch_idle": 12, "blocks_per_sm": 0, "stack": 40, "ms": 1.234}
// so it can be read and rewritten line by line and still parsed as JSON.

static bool key_ok(const char *key)
{
    if (!key || !*key) return false;
    for (const char *c = key; *c; ++c)
        if (*c == '"' || *c == '\\' || *c == '\n' || *c == '\r' || (unsigned char)*c < 0x20) return false;
    return true;
}

static std::vector<std::string> read_entries(const char *path)
{
    std::vector<std::string> out;
    FILE *f = std::fopen(path, "r");
    if (!f) return out;
    char buf[4096];
    while (std::fgets(buf, sizeof(buf), f)) {
        std::string line(buf);
        while (!line.empty() && (line.back() == '\n' || line.back() == '\r' || line.back() == ' ' ||
                                 line.back() == ','))
            line.pop_back();
        size_t s = 0;
        while (s < line.size() && line[s] == ' ') ++s;
        if (s < line.size() && line[s] == '"') out.push_back(line.substr(s));
    }
    std::fclose(f);
    return out;
}

static bool entry_has_key(const std::string &e, const char *key)
{
    const std::string head = std::string("\"") + key + "\":";
    return e.compare(0, head.size(), head) == 0;
}

static bool entry_int(const std::string &e, const char *name, int &v)
{
    const std::string pat = std::string("\"") + name + "\":";
    const size_t p = e.find(pat);
    if (p == std::string::npos) return false;
    char *end = nullptr;
    const long x = std::strtol(e.c_str() + p + pat.size(), &end, 10);
    if (end == e.c_str() + p + pat.size()) return false;
    v = (int)x;
    return true;
}

static rta_batch_params with_param(rta_batch_params p, int dim, int value)
{
    switch (dim) {
    case 0: p.digit_bits = value; break;
    case 1: p.fetch_idle = value; break;
    case 2: p.blocks_per_sm = value; break;
    default: p.stack = value; break;
    }
    return p;
}

extern "C" {

int rta_tune_cache_lookup(const char *path, const char *key, rta_batch_params *p)
{
    if (!path || !p || !key_ok(key)) return RTA_ERR_INVALID;
    for (const std::string &e : read_entries(path)) {
        if (!entry_has_key(e, key)) continue;
        rta_batch_params q;
        if (entry_int(e, "digit_bits", q.digit_bits) && entry_int(e, "fetch_idle", q.fetch_idle) &&
            entry_int(e, "blocks_per_sm", q.blocks_per_sm) && entry_int(e, "stack", q.stack) && valid_params(q)) {
            *p = q;
            return RTA_OK;
        }
        return RTA_ERR_INVALID;
    }
    return RTA_ERR_INVALID;
}

int rta_tune_cache_store(const char *path, const char *key, const rta_batch_params *p, float ms)
{
    if (!path || !p || !key_ok(key) || !valid_params(*p)) return RTA_ERR_INVALID;
    std::vector<std::string> entries;
    for (const std::string &e : read_entries(path))
        if (!entry_has_key(e, key)) entries.push_back(e);
    char line[1024];
    std::snprintf(line, sizeof(line),
                  "\"%s\": {\"digit_bits\": %d, \"fetch_idle\": %d, \"blocks_per_sm\": %d, \"stack\": %d, "
                  "\"ms\": %.6g}",
                  key, p->digit_bits, p->fetch_idle, p->blocks_per_sm, p->stack, (double)ms);
    entries.push_back(line);
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "w");
    if (!f) {
        set_error_message("rta_tune_cache_store: cannot write the cache file");
        return RTA_ERR_INVALID;
    }
    std::fputs("{\n", f);
    for (size_t i = 0; i < entries.size(); ++i) {
        std::fputs(entries[i].c_str(), f);
        std::fputs(i + 1 < entries.size() ? ",\n" : "\n", f);
    }
    std::fputs("}\n", f);
    const bool ok = std::fclose(f) == 0 && std::rename(tmp.c_str(), path) == 0;
    if (!ok) {
        set_error_message("rta_tune_cache_store: cannot replace the cache file");
        return RTA_ERR_INVALID;
    }
    return RTA_OK;
}

int rta_batch_tune_key(const rta_batch *b, char *buf, uint32_t size)
{
    if (!b || !buf || size == 0 || b->meshes == 0) return RTA_ERR_INVALID;
    int dev = 0;
    cudaDeviceProp prop;
    RTA_CUDA_TRY(cudaGetDevice(&dev));
    RTA_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    std::string name(prop.name);
    for (char &c : name)
        if (c == '"' || c == '\\' || (unsigned char)c < 0x20) c = '_';
    int tl = 0, rl = 0;
    while ((1ull << tl) < b->n) ++tl;
    while ((1ull << rl) < (uint64_t)b->rays) ++rl;
    const int w = std::snprintf(buf, size, "%s|sm%d|meshes%u|tris2^%d|rays2^%d", name.c_str(),
                                prop.multiProcessorCount, b->meshes, tl, rl);
    return (w > 0 && (uint32_t)w < size) ? RTA_OK : RTA_ERR_INVALID;
}

int rta_batch_autotune(rta_batch *b, const void *tris, const float *orig, const float *dir, const float *maxt,
                       void *hits, const char *cache_path, int reps, rta_stream_t stream,
                       rta_batch_params *chosen, float *best_ms)
{
    if (!b || !tris || b->meshes == 0 || reps < 1) return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    char key[512];
    int rc = rta_batch_tune_key(b, key, sizeof(key));
    if (rc) return rc;
    rta_batch_params cached;
    if (cache_path && rta_tune_cache_lookup(cache_path, key, &cached) == RTA_OK &&
        sort_passes(30 + (int)b->mesh_bits, cached.digit_bits) <= kMaxPasses) {
        b->params = cached;
        if (chosen) *chosen = cached;
        if (best_ms) *best_ms = -1.0f;   // taken from the cache, not timed
        return RTA_OK;
    }
    cudaEvent_t e0, e1;
    RTA_CUDA_TRY(cudaEventCreate(&e0));
    RTA_CUDA_TRY(cudaEventCreate(&e1));
    auto time_params = [&](const rta_batch_params &p, float &ms) -> int {
        b->params = p;
        int r = rta_batch_run(b, tris, orig, dir, maxt, hits, stream);   // captures the graph
        if (r) return r;
        RTA_CUDA_TRY(cudaStreamSynchronize(s));
        std::vector<float> t;
        for (int i = 0; i < reps; ++i) {
            RTA_CUDA_TRY(cudaEventRecord(e0, s));
            if ((r = rta_batch_run(b, tris, orig, dir, maxt, hits, stream))) return r;
            RTA_CUDA_TRY(cudaEventRecord(e1, s));
            RTA_CUDA_TRY(cudaEventSynchronize(e1));
            float x = 0.f;
            RTA_CUDA_TRY(cudaEventElapsedTime(&x, e0, e1));
            t.push_back(x);
        }
        std::sort(t.begin(), t.end());
        ms = t[t.size() / 2];
        return RTA_OK;
    };
    const int max_bps = batch_trace_max_blocks_per_sm(40);
    const std::vector<std::vector<int>> cand = {
        {8, 9, 10, 11}, {4, 8, 12, 16, 24}, {0, std::max(1, max_bps / 2), std::max(1, (3 * max_bps) / 4)}, {40, 64}};
    rta_batch_params best = b->params;
    if (sort_passes(30 + (int)b->mesh_bits, best.digit_bits) > kMaxPasses) best.digit_bits = 8;
    float best_t = 0.f;
    rc = time_params(best, best_t);
    for (int dim = 0; dim < 4 && !rc; ++dim) {
        for (int v : cand[dim]) {
            rta_batch_params p = with_param(best, dim, v);
            if (std::memcmp(&p, &best, sizeof(p)) == 0) continue;
            if (sort_passes(30 + (int)b->mesh_bits, p.digit_bits) > kMaxPasses) continue;
            float t = 0.f;
            if ((rc = time_params(p, t))) break;
            if (t < best_t) {
                best_t = t;
                best = p;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    b->params = best;
    if (chosen) *chosen = best;
    if (best_ms) *best_ms = best_t;
    if (cache_path) return rta_tune_cache_store(cache_path, key, &best, best_t);
    return RTA_OK;
}

} // extern "C"
