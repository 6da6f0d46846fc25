// build.cu -- LBVH construction on sm_103a.
//
// Pipeline (one stream, no host synchronisation, seven kernels + one memset):
//   memset   sort histograms, tile counters, look-back words, refit list count
//   bounds   positions -> centroids, scene box (last-block reduction)
//            [initTriangles + calculateVoxelBounds, lbvh-kernels.cu:344-359, 496-535]
//   morton   centroids -> codes, digit histograms of every sort pass
//            [morton_codes2, lbvh-kernels.cu:169-183, 405-421]
//   sort x P onesweep LSD radix passes (8-, 10- or 11-bit digits, decoupled
//            look-back)
//            [thrust::sort_by_key, lbvh-kernels.cu:537-555]
//   karras   radix-tree links + parent links; Morton-ordered triangles
//            [build_tree_karras, :186-256; permutation, :557-578]
//   refit    node boxes as unions over Morton ranges, equal-code leaf
//            collapse (three kernels: segments, their summary, the nodes
//            that cross segment borders)
//            [build_bounding_boxes_karras2, :258-341]
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "lbvh.cuh"

namespace rta {

// ------------------------------------------------------------------------- //
// host error state                                                           //
// ------------------------------------------------------------------------- //

static thread_local std::string g_last_error;

void set_cuda_error(cudaError_t e, const char *where)
{
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
}

void set_error_message(const char *msg) { g_last_error = msg; }

int check_launch(const char *where)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_cuda_error(e, where);
        return RTA_ERR_CUDA;
    }
    return RTA_OK;
}

static int num_sms()
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

__global__ void __launch_bounds__(kBoundsThreads)
k_bounds(const float *__restrict__ tris, uint32_t n, float *__restrict__ cent,
         float *__restrict__ partial, BuildState *__restrict__ st, uint32_t *__restrict__ flags,
         float grid)
{
    pdl_enter();
    // init +-1e11 as calculateVoxelBounds does (lbvh-kernels.cu:519-520)
    float lo[3] = {100000000000.0f, 100000000000.0f, 100000000000.0f};
    float hi[3] = {-100000000000.0f, -100000000000.0f, -100000000000.0f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float a[3], b[3], c[3];
        load_positions(tris + (size_t)i * kTriFloats, a, b, c);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // aabbOfTri (:141-153), then the reduce_max functor (:496-516)
            lo[k] = ref_min(lo[k], ref_min(ref_min(a[k], b[k]), c[k]));
            hi[k] = ref_max(hi[k], ref_max(ref_max(a[k], b[k]), c[k]));
            // center_of_gravity (:60-63): ((a+b)+c)/3.0f
            float s = __fadd_rn(__fadd_rn(a[k], b[k]), c[k]);
            cent[(size_t)i * 3 + k] = __fdiv_rn(s, 3.0f);
        }
    }
    // block reduction
#pragma unroll
    for (int off = 16; off; off >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = ref_min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = ref_max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    __shared__ float s_box[kBoundsThreads / 32][6];
    __shared__ bool s_last;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 3; ++k) { s_box[w][k] = lo[k]; s_box[w][3 + k] = hi[k]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 1; j < kBoundsThreads / 32; ++j)
            for (int k = 0; k < 3; ++k) {
                lo[k] = ref_min(lo[k], s_box[j][k]);
                hi[k] = ref_max(hi[k], s_box[j][3 + k]);
            }
        for (int k = 0; k < 3; ++k) {
            partial[blockIdx.x * 6 + k] = lo[k];
            partial[blockIdx.x * 6 + 3 + k] = hi[k];
        }
        __threadfence();
        uint32_t ticket = atomicAdd(&st->done, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    // the last block folds every block's box
    __threadfence();
    float l2[3] = {100000000000.0f, 100000000000.0f, 100000000000.0f};
    float h2[3] = {-100000000000.0f, -100000000000.0f, -100000000000.0f};
    for (uint32_t j = threadIdx.x; j < gridDim.x; j += blockDim.x)
        for (int k = 0; k < 3; ++k) {
            l2[k] = ref_min(l2[k], __ldcg(partial + j * 6 + k));
            h2[k] = ref_max(h2[k], __ldcg(partial + j * 6 + 3 + k));
        }
#pragma unroll
    for (int off = 16; off; off >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            l2[k] = ref_min(l2[k], __shfl_xor_sync(0xffffffffu, l2[k], off));
            h2[k] = ref_max(h2[k], __shfl_xor_sync(0xffffffffu, h2[k], off));
        }
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < 3; ++k) { s_box[w][k] = l2[k]; s_box[w][3 + k] = h2[k]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 1; j < kBoundsThreads / 32; ++j)
            for (int k = 0; k < 3; ++k) {
                l2[k] = ref_min(l2[k], s_box[j][k]);
                h2[k] = ref_max(h2[k], s_box[j][3 + k]);
            }
        uint32_t fl = 0;
        for (int k = 0; k < 3; ++k) {
            st->lo[k] = l2[k];
            st->hi[k] = h2[k];
            // d = GRIDSIZE/(max - min), computed on the host in the reference (:414-417)
            float d = __fdiv_rn(grid, __fsub_rn(h2[k], l2[k]));
            st->scale[k] = d;
            if (!isfinite(d)) fl |= RTA_DEV_ZERO_EXTENT;
        }
        if (fl) atomicOr(flags, fl);
        st->done = 0;   // ready for the next build
    }
}

// ------------------------------------------------------------------------- //
// kernel: Morton codes + digit histograms                                    //
// ------------------------------------------------------------------------- //

// codes of every triangle plus the digit histograms of all `passes` sort
// passes (digit width dbits) in dynamic shared memory, folded once per block
// 1024-thread blocks, two per SM: fewer blocks fold fewer shared histograms
// into the global ones (1M 30-bit build 0.2055 -> 0.2034 ms; 256 threads at
// 2, 4 or 8 blocks per SM, 512 at 2 and 1024 at 1 were slower or level)
#ifndef RTA_MORTON_THREADS
#define RTA_MORTON_THREADS 1024
#endif
#ifndef RTA_MORTON_BLOCKS_PER_SM
#define RTA_MORTON_BLOCKS_PER_SM 2
#endif
template <typename Key, int DBITS>
__global__ void __launch_bounds__(RTA_MORTON_THREADS)
k_morton(const float *__restrict__ cent, uint32_t n, Key *__restrict__ keys,
         const BuildState *__restrict__ st, SortScratchHeader *__restrict__ hdr,
         uint32_t *__restrict__ flags, int passes, uint32_t grid_mask)
{
    pdl_enter();
    extern __shared__ uint32_t s_hist[];
    constexpr int radix = 1 << DBITS;
    for (int j = threadIdx.x; j < passes * radix; j += blockDim.x) s_hist[j] = 0;
    __syncthreads();
    const float lo[3] = {st->lo[0], st->lo[1], st->lo[2]};
    const float d[3] = {st->scale[0], st->scale[1], st->scale[2]};
    bool wrapped = false;
    // (one atomic per run of equal digits in a warp, found by shuffles and
    // ballots, measured slower: 4M 63-bit 36.5 -> 65.5 us)
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float c[3] = {cent[(size_t)i * 3 + 0], cent[(size_t)i * 3 + 1], cent[(size_t)i * 3 + 2]};
        Key k = (Key)morton_code(c, lo, d, grid_mask, wrapped);
        keys[i] = k;
        hist_add<DBITS>(s_hist, k, passes);
    }
    if (__any_sync(0xffffffffu, wrapped) && (threadIdx.x & 31) == 0) atomicOr(flags, RTA_DEV_QUANT_WRAP);
    __syncthreads();
    for (int j = threadIdx.x; j < passes * radix; j += blockDim.x)
        if (s_hist[j]) atomicAdd(hdr->hist + j, s_hist[j]);
}

template <typename Key, int DBITS>
static cudaError_t morton_launch_db(int mb, int mt, size_t hsmem, cudaStream_t s, const float *cent, uint32_t n,
                                    void *keys, const BuildState *st, SortScratchHeader *hdr, uint32_t *flags,
                                    int passes, uint32_t gmask)
{
    static bool smem_set = false;
    if (!smem_set) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_morton<Key, DBITS>, cudaFuncAttributeMaxDynamicSharedMemorySize, 48 * 1024);
        if (e != cudaSuccess) return e;
        smem_set = true;
    }
    return launch_pdl(true, k_morton<Key, DBITS>, dim3(mb), dim3(mt), hsmem, s, cent, n, (Key *)keys, st, hdr, flags,
                      passes, gmask);
}

// the Morton kernel for digit width db (8 to 11)
template <typename Key>
static cudaError_t morton_launch(int db, int mb, int mt, size_t hsmem, cudaStream_t s, const float *cent,
                                 uint32_t n, void *keys, const BuildState *st, SortScratchHeader *hdr,
                                 uint32_t *flags, int passes, uint32_t gmask)
{
    switch (db) {
    case 9: return morton_launch_db<Key, 9>(mb, mt, hsmem, s, cent, n, keys, st, hdr, flags, passes, gmask);
    case 10: return morton_launch_db<Key, 10>(mb, mt, hsmem, s, cent, n, keys, st, hdr, flags, passes, gmask);
    case 11: return morton_launch_db<Key, 11>(mb, mt, hsmem, s, cent, n, keys, st, hdr, flags, passes, gmask);
    default: return morton_launch_db<Key, 8>(mb, mt, hsmem, s, cent, n, keys, st, hdr, flags, passes, gmask);
    }
}

// ------------------------------------------------------------------------- //
// kernel: Karras radix tree + Morton-ordered triangles                        //
// ------------------------------------------------------------------------- //

template <typename Key>
__global__ void __launch_bounds__(256)
k_karras(const Key *__restrict__ codes, const uint32_t *__restrict__ ids, uint32_t n,
         uint4 *__restrict__ links, uint32_t *__restrict__ parents,
         const float *__restrict__ tris_in, float *__restrict__ tris_out, TriRec *__restrict__ tris_rec)
{
    pdl_enter();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // with tris_rec: the 48-byte triangle of sorted position i (its gather
    // overlaps the split search)
    TriRec tr;
    if (tris_rec) {
        const uint32_t id = __ldg(ids + i);
        tr = make_tri(tris_in + (size_t)id * kTriFloats, id);
    }
    if (i + 1 < n) karras_node(codes, n, i, links, parents);
    if (tris_rec) tris_rec[i] = tr;
    // invert_triangle_permutation_cuda (:557-578): the 104-byte records in
    // Morton order, when asked for (the 48-byte triangles are gathered above)
    if (tris_out) {
        const uint32_t id = __ldg(ids + i);
        const float *src = tris_in + (size_t)id * kTriFloats;
        const float2 *s2 = reinterpret_cast<const float2 *>(src);
        float2 *d2 = reinterpret_cast<float2 *>(tris_out + (size_t)i * kTriFloats);
#pragma unroll
        for (int j = 0; j < kTriFloats / 2; ++j) d2[j] = __ldg(s2 + j);
    }
}

// ------------------------------------------------------------------------- //
// kernel: the bounded-wait self-test                                           //
// ------------------------------------------------------------------------- //

// Tile 1's look-back for 32 counters whose tile-0 words stay zero ("not
// written yet"): each lane polls to the limit, raises the timeout flag and
// returns.
__global__ void k_selftest_wait(const uint32_t *__restrict__ stat, uint32_t *__restrict__ flags)
{
    (void)lookback(stat + threadIdx.x, 32u, 1u, flags);
}

// ------------------------------------------------------------------------- //
// kernel: write the reference 2F4 node array (dumps and parity checks)       //
// ------------------------------------------------------------------------- //

__global__ void k_to_2f4(const NodeRec *__restrict__ nodes, const RootRec *__restrict__ root,
                         const uint32_t *__restrict__ parents, const TriRec *__restrict__ tris,
                         uint32_t n, float4 *__restrict__ out)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 2 * n - 1) return;
    float lo[3], hi[3];
    uint32_t link;   // this node's link as seen from its parent (or the root record)
    if (k != 0 && parent_index(parents[k]) >= n - 1) {   // only a broken build gets here
        out[2 * k + 0] = make_float4(0.f, 0.f, 0.f, 0.f);
        out[2 * k + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (k == 0) {
        for (int a = 0; a < 3; ++a) { lo[a] = root->lo[a]; hi[a] = root->hi[a]; }
        link = root->link;
    } else {
        const uint32_t pl = parents[k];
        const NodeRec *nd = nodes + parent_index(pl);
        const float *f = reinterpret_cast<const float *>(nd);
        for (int a = 0; a < 3; ++a) {
            lo[a] = f[slot_lo(pl & 1u, a)];
            hi[a] = f[slot_hi(pl & 1u, a)];
        }
        link = reinterpret_cast<const uint32_t *>(&nd->q3)[pl & 1u];
    }
    uint32_t w0, w1;
    if (k >= n - 1) {
        w0 = 1u << 1;           // original leaves keep (tris = k-(n-1), elems = 1)
        w1 = k - (n - 1);
    } else if (is_leaf(link)) {  // a collapsed inner node
        // its count is its own range's size, the sum of its children's
        // sizes (the link's count field saturates at 64, and the triangle
        // record keeps only the largest collapsed count starting at that
        // leaf, which a collapsed node nested in a larger one does not have)
        const uint4 q = nodes[k].q3;
        w0 = (q.z + q.w) << 1;
        w1 = leaf_first(link);
    } else {
        // reference numbering of the children: an inner link is the node
        // index; a leaf link (first, count) is leaf n-1+first if count is 1,
        // else a collapsed inner node, which is its range's end for a left
        // child and its range's start for a right child
        const uint4 q = nodes[k].q3;
        const uint32_t l = !is_leaf(q.x) ? q.x : (q.z == 1u ? n - 1 + leaf_first(q.x) : leaf_first(q.x) + q.z - 1u);
        const uint32_t r = !is_leaf(q.y) ? q.y : (q.w == 1u ? n - 1 + leaf_first(q.y) : leaf_first(q.y));
        w0 = (l << 1) | 1u;
        w1 = r;
    }
    out[2 * k + 0] = make_float4(__uint_as_float(w0), __uint_as_float(w1), lo[0], lo[1]);
    out[2 * k + 1] = make_float4(lo[2], hi[0], hi[1], hi[2]);
}

} // namespace rta

// ------------------------------------------------------------------------- //
// host side                                                                  //
// ------------------------------------------------------------------------- //

using namespace rta;

struct rta_lbvh_ctx {
    uint32_t cap = 0;
    int bits = 0;
    int digit_bits = 8;   // radix digit width of the sort (8 to 11)
    // device buffers
    void *keys0 = nullptr, *keys1 = nullptr;
    uint32_t *vals0 = nullptr, *vals1 = nullptr;
    float *cent = nullptr;
    float *partial = nullptr;
    BuildState *state = nullptr;
    unsigned char *scratch = nullptr;   // SortScratchHeader + tile status words
    size_t scratch_bytes = 0;
    NodeRec *nodes = nullptr;
    RootRec *root = nullptr;
    uint32_t *parents = nullptr;
    uint32_t *counters = nullptr;   // refit: the inner nodes that cross a segment border
    uint4 *links = nullptr;         // Karras links per inner node, read by the refit
    TriRec *tris = nullptr;
    uint32_t *status = nullptr;
    float *rbox = nullptr;   // refit tables: prefix and suffix unions, t1, t2
    // last build
    uint32_t n = 0;
    int last_bits = 30;
    void *codes = nullptr;       // sorted keys (keys0 or keys1)
    uint32_t *index = nullptr;   // sorted ids (vals0 or vals1)
    // recorded on the build's stream after each build's last kernel: work on
    // other streams that reads the tree waits for it (rta_lbvh::ready)
    cudaEvent_t built = nullptr;
    // per-pass timing (rta_lbvh_set_timing): events before the first pass
    // and after each of the RTA_LBVH_PASSES passes of the last build
    bool timing = false, timed = false;
    cudaEvent_t pass_ev[RTA_LBVH_PASSES + 1] = {};
};

// four blocks per SM, each looping over triangles, then one fold of their
// boxes: 1M build 0.186 -> 0.184 ms, 4M 0.748 -> 0.745 ms against eight
// (16 and 32 level or slower)
#ifndef RTA_BOUNDS_BLOCKS_PER_SM
#define RTA_BOUNDS_BLOCKS_PER_SM 4
#endif
static int bounds_blocks(uint32_t n)
{
    int want = (int)((n + kBoundsThreads - 1) / kBoundsThreads);
    int cap = num_sms() * RTA_BOUNDS_BLOCKS_PER_SM;
    return want < cap ? (want > 0 ? want : 1) : cap;
}

static bool valid_digit_bits(int b) { return b >= 8 && b <= 11; }


// tile status words per tile, the most any supported digit width needs
static size_t status_words_per_tile(int key_bits)
{
    size_t w = 0;
    for (int b : {8, 9, 10, 11}) {
        size_t v = (size_t)sort_passes(key_bits, b) << b;
        if (v > w) w = v;
    }
    return w;
}

static void free_ctx(rta_lbvh_ctx *c)
{
    void *ptrs[] = {c->keys0, c->keys1, c->vals0, c->vals1, c->cent,    c->partial, c->state, c->scratch,
                    c->nodes, c->root,  c->parents, c->counters, c->tris, c->status,  c->rbox, c->links};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    // the settings and events outlive the buffers
    rta_lbvh_ctx keep;
    keep.digit_bits = c->digit_bits;
    keep.built = c->built;
    keep.timing = c->timing;
    for (int k = 0; k <= RTA_LBVH_PASSES; ++k) keep.pass_ev[k] = c->pass_ev[k];
    *c = keep;
}

template <typename Key>
static int sort_keys(rta_lbvh_ctx *c, uint32_t n, int passes, SortScratchHeader *hdr, uint32_t *tstat,
                     cudaStream_t s)
{
    Key *ks = nullptr;
    uint32_t *vs = nullptr;
    int rc;
    Key *k0 = (Key *)c->keys0, *k1 = (Key *)c->keys1;
    switch (c->digit_bits) {
    case 9:
        rc = sort_passes_launch<Key, 9>(k0, k1, c->vals0, c->vals1, n, passes, hdr, tstat, c->status, nullptr,
                                        0u, s, &ks, &vs, true);
        break;
    case 10:
        rc = sort_passes_launch<Key, 10>(k0, k1, c->vals0, c->vals1, n, passes, hdr, tstat, c->status, nullptr,
                                         0u, s, &ks, &vs, true);
        break;
    case 11:
        rc = sort_passes_launch<Key, 11>(k0, k1, c->vals0, c->vals1, n, passes, hdr, tstat, c->status, nullptr,
                                         0u, s, &ks, &vs, true);
        break;
    default:
        rc = sort_passes_launch<Key, 8>(k0, k1, c->vals0, c->vals1, n, passes, hdr, tstat, c->status, nullptr,
                                        0u, s, &ks, &vs, true);
    }
    c->codes = ks;
    c->index = vs;
    return rc;
}

extern "C" {

const char *rta_last_error(void) { return g_last_error.c_str(); }

uint32_t rta_lbvh_max_triangles(void) { return kMaxTriangles; }

int rta_lbvh_create(rta_lbvh_ctx **ctx)
{
    if (!ctx) return RTA_ERR_INVALID;
    *ctx = new rta_lbvh_ctx();
    return RTA_OK;
}

int rta_lbvh_destroy(rta_lbvh_ctx *ctx)
{
    if (!ctx) return RTA_ERR_INVALID;
    free_ctx(ctx);
    if (ctx->built) cudaEventDestroy(ctx->built);
    for (cudaEvent_t e : ctx->pass_ev)
        if (e) cudaEventDestroy(e);
    delete ctx;
    return RTA_OK;
}

int rta_lbvh_set_digit_bits(rta_lbvh_ctx *c, int digit_bits)
{
    if (!c || !valid_digit_bits(digit_bits)) return RTA_ERR_INVALID;
    c->digit_bits = digit_bits;
    return RTA_OK;
}

int rta_lbvh_reserve(rta_lbvh_ctx *c, uint32_t n, int bits)
{
    if (!c || n == 0 || n > kMaxTriangles || (bits != 30 && bits != 63)) return RTA_ERR_INVALID;
    if (n <= c->cap && (bits == 30 || c->bits == 63)) return RTA_OK;
    free_ctx(c);
    const size_t ksz = bits == 63 ? 8 : 4;
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    c->scratch_bytes = sizeof(SortScratchHeader) + status_words_per_tile(bits) * tiles * 4;
    RTA_CUDA_TRY(cudaMalloc(&c->keys0, (size_t)n * ksz));
    RTA_CUDA_TRY(cudaMalloc(&c->keys1, (size_t)n * ksz));
    RTA_CUDA_TRY(cudaMalloc(&c->vals0, (size_t)n * 4));
    RTA_CUDA_TRY(cudaMalloc(&c->vals1, (size_t)n * 4));
    RTA_CUDA_TRY(cudaMalloc(&c->cent, (size_t)n * 12));
    RTA_CUDA_TRY(cudaMalloc(&c->partial, (size_t)bounds_blocks(n) * 6 * 4));
    RTA_CUDA_TRY(cudaMalloc(&c->state, sizeof(BuildState)));
    RTA_CUDA_TRY(cudaMemset(c->state, 0, sizeof(BuildState)));
    RTA_CUDA_TRY(cudaMalloc(&c->scratch, c->scratch_bytes));
    RTA_CUDA_TRY(cudaMalloc(&c->nodes, (size_t)(n > 1 ? n - 1 : 1) * sizeof(NodeRec)));
    RTA_CUDA_TRY(cudaMalloc(&c->root, sizeof(RootRec)));
    RTA_CUDA_TRY(cudaMalloc(&c->parents, (size_t)(2 * n - 1) * 4));
    RTA_CUDA_TRY(cudaMalloc(&c->counters, (size_t)n * 4));
    RTA_CUDA_TRY(cudaMalloc(&c->links, (size_t)n * sizeof(uint4)));
    RTA_CUDA_TRY(cudaMalloc(&c->tris, (size_t)n * sizeof(TriRec)));
    RTA_CUDA_TRY(cudaMalloc(&c->status, 64));
    RTA_CUDA_TRY(cudaMemset(c->status, 0, 64));
    RTA_CUDA_TRY(cudaMalloc(&c->rbox, refit_layout(n).total * 6 * sizeof(float)));
    c->cap = n;
    c->bits = bits;
    return RTA_OK;
}

int rta_lbvh_build(rta_lbvh_ctx *c, const void *tris, uint32_t n, int bits, void *tris_out,
                   rta_stream_t stream)
{
    if (!c || !tris || n == 0 || n > kMaxTriangles || (bits != 30 && bits != 63))
        return RTA_ERR_INVALID;
    int rc = rta_lbvh_reserve(c, n, bits);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int db = c->digit_bits;
    const int passes = sort_passes(bits == 63 ? 63 : 30, db);
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    SortScratchHeader *hdr = reinterpret_cast<SortScratchHeader *>(c->scratch);
    uint32_t *tstat = reinterpret_cast<uint32_t *>(c->scratch + sizeof(SortScratchHeader));
    const size_t used = sizeof(SortScratchHeader) + ((size_t)passes << db) * tiles * 4;
    RTA_CUDA_TRY(cudaMemsetAsync(c->scratch, 0, used, s));
    // per-pass events (only with timing on; they end the launches' overlap
    // at the pass borders)
    auto mark = [&](int k) -> int {
        if (c->timing) RTA_CUDA_TRY(cudaEventRecord(c->pass_ev[k], s));
        return RTA_OK;
    };
    c->timed = false;
    if ((rc = mark(0))) return rc;

    const float *tin = static_cast<const float *>(tris);
    const int bb = bounds_blocks(n);
    k_bounds<<<bb, kBoundsThreads, 0, s>>>(tin, n, c->cent, c->partial, c->state, c->status,
                                           bits == 63 ? 2097152.0f : 1024.0f);
    if ((rc = check_launch("k_bounds"))) return rc;
    if ((rc = mark(1))) return rc;
    const int eb = (int)((n + 255) / 256);
    const int mt = RTA_MORTON_THREADS, mcap = num_sms() * RTA_MORTON_BLOCKS_PER_SM;
    const int mb = (int)((n + mt - 1) / mt) < mcap ? (int)((n + mt - 1) / mt) : mcap;
    const uint32_t gmask = bits == 63 ? 0x1fffffu : 0x3ffu;
    const size_t hsmem = ((size_t)passes << db) * 4;
    RTA_CUDA_TRY(bits == 63 ? morton_launch<uint64_t>(db, mb, mt, hsmem, s, c->cent, n, c->keys0, c->state, hdr,
                                                      c->status, passes, gmask)
                            : morton_launch<uint32_t>(db, mb, mt, hsmem, s, c->cent, n, c->keys0, c->state, hdr,
                                                      c->status, passes, gmask));

    if ((rc = mark(2))) return rc;
    rc = bits == 63 ? sort_keys<uint64_t>(c, n, passes, hdr, tstat, s)
                    : sort_keys<uint32_t>(c, n, passes, hdr, tstat, s);
    if (rc) return rc;
    if ((rc = mark(3))) return rc;
    TriRec *kg = RTA_KARRAS_GATHER ? c->tris : nullptr;
    RTA_CUDA_TRY(bits == 63 ? launch_pdl(true, k_karras<uint64_t>, dim3(eb), dim3(256), 0, s,
                                         (const uint64_t *)c->codes, (const uint32_t *)c->index, n, c->links,
                                         c->parents, tin, (float *)tris_out, kg)
                            : launch_pdl(true, k_karras<uint32_t>, dim3(eb), dim3(256), 0, s,
                                         (const uint32_t *)c->codes, (const uint32_t *)c->index, n, c->links,
                                         c->parents, tin, (float *)tris_out, kg));
    if ((rc = mark(4))) return rc;
    const uint32_t cap = n > 1 ? n - 1 : 1;
    rc = bits == 63 ? refit_launch<uint64_t, false>((const uint64_t *)c->codes, n, nullptr, nullptr, kg ? nullptr : tin, c->index,
                                                    c->nodes, c->links, c->parents, c->tris, c->root, c->rbox, c->counters,
                                                    cap, &hdr->n_cross, &hdr->refit_ticket, c->status, num_sms(), s,
                                                    true)
                    : refit_launch<uint32_t, false>((const uint32_t *)c->codes, n, nullptr, nullptr, kg ? nullptr : tin, c->index,
                                                    c->nodes, c->links, c->parents, c->tris, c->root, c->rbox, c->counters,
                                                    cap, &hdr->n_cross, &hdr->refit_ticket, c->status, num_sms(), s,
                                                    true);
    if (rc) return rc;
    if ((rc = mark(5))) return rc;
    c->timed = c->timing;
    if (!c->built) RTA_CUDA_TRY(cudaEventCreateWithFlags(&c->built, cudaEventDisableTiming));
    RTA_CUDA_TRY(cudaEventRecord(c->built, s));
    c->n = n;
    c->last_bits = bits;
    return RTA_OK;
}

int rta_lbvh_set_timing(rta_lbvh_ctx *c, int on)
{
    if (!c) return RTA_ERR_INVALID;
    if (on && !c->pass_ev[0])
        for (cudaEvent_t &e : c->pass_ev) RTA_CUDA_TRY(cudaEventCreate(&e));
    c->timing = on != 0;
    c->timed = false;
    return RTA_OK;
}

int rta_lbvh_pass_ms(rta_lbvh_ctx *c, float *ms)
{
    if (!c || !ms || !c->timed) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaEventSynchronize(c->pass_ev[RTA_LBVH_PASSES]));
    for (int k = 0; k < RTA_LBVH_PASSES; ++k)
        RTA_CUDA_TRY(cudaEventElapsedTime(&ms[k], c->pass_ev[k], c->pass_ev[k + 1]));
    return RTA_OK;
}

int rta_lbvh_get(const rta_lbvh_ctx *c, rta_lbvh *out)
{
    if (!c || !out || c->n == 0) return RTA_ERR_INVALID;
    out->nodes = c->nodes;
    out->root = c->root;
    out->tris = c->tris;
    out->index = c->index;
    out->codes = c->codes;
    out->parents = c->parents;
    out->n = c->n;
    out->morton_bits = c->last_bits;
    out->status = c->status;
    out->ready = c->built;
    return RTA_OK;
}

int rta_lbvh_status(const rta_lbvh *bvh, rta_stream_t stream, uint32_t *flags)
{
    if (!bvh || !flags) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    RTA_CUDA_TRY(cudaMemcpy(flags, bvh->status, 4, cudaMemcpyDeviceToHost));
    return RTA_OK;
}

int rta_selftest_bounded_wait(rta_stream_t stream, uint32_t *flags)
{
    if (!flags) return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *d = nullptr;   // [0]: flags, [1 .. 32]: tile 0's status words (never written)
    RTA_CUDA_TRY(cudaMalloc(&d, 33 * 4));
    cudaError_t e = cudaMemsetAsync(d, 0, 33 * 4, s);
    if (e == cudaSuccess) {
        k_selftest_wait<<<1, 32, 0, s>>>(d + 1, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpy(flags, d, 4, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_cuda_error(e, "rta_selftest_bounded_wait");
        return RTA_ERR_CUDA;
    }
    return RTA_OK;
}

int rta_lbvh_to_2f4(const rta_lbvh *bvh, void *nodes_2f4, rta_stream_t stream)
{
    if (!bvh || !nodes_2f4 || bvh->n == 0) return RTA_ERR_INVALID;
    const uint32_t total = 2 * bvh->n - 1;
    k_to_2f4<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        (const NodeRec *)bvh->nodes, (const RootRec *)bvh->root, bvh->parents,
        (const TriRec *)bvh->tris, bvh->n, (float4 *)nodes_2f4);
    return check_launch("k_to_2f4");
}

} // extern "C"
