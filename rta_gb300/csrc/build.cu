// build.cu -- LBVH construction on sm_103a.
//
// Pipeline (one stream, no host synchronisation, five kernels + one memset):
//   memset   sort histograms, tile counters and look-back words
//   bounds   positions -> centroids, scene box (last-block reduction)
//            [initTriangles + calculateVoxelBounds, lbvh-kernels.cu:344-359, 496-535]
//   morton   centroids -> codes, digit histograms of every sort pass
//            [morton_codes2, lbvh-kernels.cu:169-183, 405-421]
//   sort x P onesweep LSD radix passes (8-bit digits, decoupled look-back)
//            [thrust::sort_by_key, lbvh-kernels.cu:537-555]
//   karras   radix-tree links + parent links; Morton-ordered triangles
//            [build_tree_karras, :186-256; permutation, :557-578]
//   refit    bottom-up boxes with equal-code leaf collapse
//            [build_bounding_boxes_karras2, :258-341]
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

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

// ------------------------------------------------------------------------- //
// build state                                                                //
// ------------------------------------------------------------------------- //

constexpr int kTriFloats = 26;         // cuda::simple_triangle = 104 bytes
constexpr int kBoundsThreads = 256;
constexpr int kSortThreads = 256;      // 8 warps
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per tile
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;

struct BuildState {
    float lo[3], hi[3], scale[3];
    uint32_t done;                 // bounds last-block ticket (self-resetting)
};

// zeroed by one memset before every build
struct SortScratchHeader {
    uint32_t hist[kMaxPasses][kRadix];
    uint32_t tile_ctr[kMaxPasses];
};

// ------------------------------------------------------------------------- //
// kernel: triangle positions -> centroids + scene box                        //
// ------------------------------------------------------------------------- //

__device__ __forceinline__ void load_positions(const float *__restrict__ t, float a[3], float b[3],
                                               float c[3])
{
    // records are 8-byte aligned (104 = 13 * 8): five 8-byte loads cover the 36
    // position bytes
    const float2 *p = reinterpret_cast<const float2 *>(t);
    float2 x0 = __ldg(p + 0), x1 = __ldg(p + 1), x2 = __ldg(p + 2), x3 = __ldg(p + 3);
    float cz = __ldg(t + 8);
    a[0] = x0.x; a[1] = x0.y; a[2] = x1.x;
    b[0] = x1.y; b[1] = x2.x; b[2] = x2.y;
    c[0] = x3.x; c[1] = x3.y; c[2] = cz;
}

__global__ void __launch_bounds__(kBoundsThreads)
k_bounds(const float *__restrict__ tris, uint32_t n, float *__restrict__ cent,
         float *__restrict__ partial, BuildState *__restrict__ st, uint32_t *__restrict__ flags,
         float grid)
{
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

// float -> unsigned as the reference's `uint x = f;` compiles on the GPU
// (cvt.rzi.u32.f32: truncation, NaN and negatives to 0, saturation)
__device__ __forceinline__ uint32_t f2u_rz_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return __float2uint_rz(v);
}

// bit k of the low 21 bits of v moves to bit 3k
__device__ __forceinline__ uint64_t spread3(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x001f00000000ffffull;
    v = (v | (v << 16)) & 0x001f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

template <typename Key>
__global__ void __launch_bounds__(256)
k_morton(const float *__restrict__ cent, uint32_t n, Key *__restrict__ keys,
         const BuildState *__restrict__ st, SortScratchHeader *__restrict__ hdr,
         uint32_t *__restrict__ flags, int passes, uint32_t grid_mask)
{
    __shared__ uint32_t s_hist[kMaxPasses * kRadix];
    for (int j = threadIdx.x; j < passes * kRadix; j += blockDim.x) s_hist[j] = 0;
    __syncthreads();
    const float lo0 = st->lo[0], lo1 = st->lo[1], lo2 = st->lo[2];
    const float d0 = st->scale[0], d1 = st->scale[1], d2 = st->scale[2];
    bool wrapped = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float *c = cent + (size_t)i * 3;
        // morton_codes2 (:174-180): center - c, times d, to unsigned, mask
        uint32_t x = f2u_rz_sat(__fmul_rn(__fsub_rn(c[0], lo0), d0));
        uint32_t y = f2u_rz_sat(__fmul_rn(__fsub_rn(c[1], lo1), d1));
        uint32_t z = f2u_rz_sat(__fmul_rn(__fsub_rn(c[2], lo2), d2));
        wrapped |= (x > grid_mask) | (y > grid_mask) | (z > grid_mask);
        uint64_t code = spread3(x & grid_mask) | (spread3(y & grid_mask) << 1) |
                        (spread3(z & grid_mask) << 2);
        Key k = (Key)code;
        keys[i] = k;
        for (int p = 0; p < passes; ++p)
            atomicAdd(&s_hist[p * kRadix + (uint32_t)((k >> (8 * p)) & 0xffu)], 1u);
    }
    if (__any_sync(0xffffffffu, wrapped) && (threadIdx.x & 31) == 0) atomicOr(flags, RTA_DEV_QUANT_WRAP);
    __syncthreads();
    for (int j = threadIdx.x; j < passes * kRadix; j += blockDim.x)
        if (s_hist[j]) atomicAdd(&hdr->hist[0][0] + j, s_hist[j]);
}

// ------------------------------------------------------------------------- //
// kernel: one onesweep LSD radix pass                                        //
// ------------------------------------------------------------------------- //
//
// A tile of 4096 keys per block: warp-level stable ranking with 8 ballots per
// key, per-warp digit counters in shared memory, decoupled look-back across
// tiles for the per-digit prefix (Merrill & Garland's single-pass scan as used
// by Adinets & Merrill's Onesweep), a shared-memory staging of the tile in
// digit order, and coalesced runs out to global memory.

template <typename Key>
struct SortSmem {
    uint32_t whist[kSortThreads / 32][kRadix];
    uint32_t digit_start[kRadix];
    uint32_t glob[kRadix];
    uint32_t scan_tmp[kSortThreads / 32];
    uint32_t tile;
    Key keys[kSortTile];
    uint32_t vals[kSortTile];
};

// block-wide exclusive scan of one value per thread (256 threads)
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *tmp)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) tmp[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < kSortThreads / 32 ? tmp[lane] : 0u;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, off);
            if (lane >= off) t += y;
        }
        if (lane < kSortThreads / 32) tmp[lane] = t;
    }
    __syncthreads();
    uint32_t before = w ? tmp[w - 1] : 0u;
    uint32_t r = before + x - v;
    __syncthreads();
    return r;
}

template <typename Key>
__global__ void __launch_bounds__(kSortThreads)
k_onesweep(const Key *__restrict__ kin, const uint32_t *__restrict__ vin, Key *__restrict__ kout,
           uint32_t *__restrict__ vout, uint32_t n, int pass, SortScratchHeader *__restrict__ hdr,
           uint32_t *__restrict__ tstat, uint32_t *__restrict__ flags)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem<Key> &S = *reinterpret_cast<SortSmem<Key> *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int shift = 8 * pass;

    if (tid == 0) S.tile = atomicAdd(&hdr->tile_ctr[pass], 1u);
    for (int j = tid; j < (kSortThreads / 32) * kRadix; j += kSortThreads) (&S.whist[0][0])[j] = 0;
    __syncthreads();
    const uint32_t tile = S.tile;
    const uint32_t base = tile * kSortTile;
    const uint32_t wbase = base + (uint32_t)w * (32 * kSortItems);

    Key k[kSortItems];
    uint32_t v[kSortItems];
    uint32_t rank[kSortItems];
    uint32_t dig[kSortItems];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = wbase + i * 32 + lane;
        bool ok = idx < n;
        k[i] = ok ? kin[idx] : (Key)~(Key)0;
        v[i] = ok ? (vin ? vin[idx] : idx) : 0u;
        dig[i] = (uint32_t)((k[i] >> shift) & 0xffu);
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t d = dig[i];
        uint32_t peers = 0xffffffffu;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            uint32_t bal = __ballot_sync(0xffffffffu, (d >> b) & 1u);
            peers &= ((d >> b) & 1u) ? bal : ~bal;
        }
        const int leader = __ffs(peers) - 1;
        uint32_t prev = 0;
        if (lane == leader) {
            prev = S.whist[w][d];
            S.whist[w][d] = prev + __popc(peers);
        }
        __syncwarp();
        prev = __shfl_sync(0xffffffffu, prev, leader);
        rank[i] = prev + __popc(peers & lt_mask);
    }
    __syncthreads();

    // per digit (thread = digit): warp offsets, tile count, block offsets
    const uint32_t d = tid;
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < kSortThreads / 32; ++j) {
        uint32_t c = S.whist[j][d];
        S.whist[j][d] = cnt;
        cnt += c;
    }
    // padding keys (beyond n) are all digit 255 and sit at the end of the last tile
    uint32_t valid = n - base < (uint32_t)kSortTile ? n - base : (uint32_t)kSortTile;
    uint32_t pad = (uint32_t)kSortTile - valid;
    uint32_t cnt_valid = (d == kRadix - 1) ? cnt - pad : cnt;

    uint32_t *my_stat = tstat + (size_t)tile * kRadix + d;
    if (tile == 0)
        st_volatile(my_stat, kStatPrefix | cnt_valid);
    else
        st_volatile(my_stat, kStatAggregate | cnt_valid);
    uint32_t start = block_excl_scan(cnt, S.scan_tmp);
    S.digit_start[d] = start;
    uint32_t gexcl = block_excl_scan(hdr->hist[pass][d], S.scan_tmp);
    uint32_t excl = 0;
    if (tile > 0) {
        excl = lookback(tstat + d, kRadix, tile, flags);
        __threadfence();
        st_volatile(my_stat, kStatPrefix | ((excl + cnt_valid) & kStatValue));
    }
    S.glob[d] = gexcl + excl - start;
    __syncthreads();

#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t pos = S.digit_start[dig[i]] + S.whist[w][dig[i]] + rank[i];
        S.keys[pos] = k[i];
        S.vals[pos] = v[i];
    }
    __syncthreads();
    for (uint32_t j = tid; j < valid; j += kSortThreads) {
        Key key = S.keys[j];
        uint32_t dst = S.glob[(uint32_t)((key >> shift) & 0xffu)] + j;
        kout[dst] = key;
        vout[dst] = S.vals[j];
    }
}

// ------------------------------------------------------------------------- //
// kernel: Karras radix tree + Morton-ordered triangles                        //
// ------------------------------------------------------------------------- //

template <typename Key> struct KeyBits;
template <> struct KeyBits<uint32_t> {
    static constexpr int tie = 32;
    __device__ static int clz(uint32_t x) { return __clz(x); }
};
template <> struct KeyBits<uint64_t> {
    static constexpr int tie = 64;
    __device__ static int clz(uint64_t x) { return __clzll(x); }
};

// common prefix length with the index tie-break (`__cpl`, :84-92)
template <typename Key>
__device__ __forceinline__ int cpl(const Key *__restrict__ codes, int n, int i, int j, Key ki)
{
    if (j < 0 || j >= n) return -1;
    Key kj = __ldg(codes + j);
    if (ki == kj) return KeyBits<Key>::tie + __clz(i ^ j);
    return KeyBits<Key>::clz(ki ^ kj);
}

template <typename Key>
__device__ __forceinline__ void karras_split(const Key *__restrict__ codes, int n, int i, int &left,
                                             int &right, int &left_size, int &right_size)
{
    // build_tree_karras (:205-249): direction, range end (exponential +
    // binary search), split (binary search with ceiling halving)
    const Key ki = __ldg(codes + i);
    int dd = cpl(codes, n, i, i + 1, ki) - cpl(codes, n, i, i - 1, ki);
    int d = dd >= 0 ? 1 : -1;
    int cpl_min = cpl(codes, n, i, i - d, ki);
    int l_max = 2;
    while (cpl(codes, n, i, i + l_max * d, ki) > cpl_min) l_max *= 2;
    int l = 0;
    for (int t = l_max / 2; t >= 1; t /= 2)
        if (cpl(codes, n, i, i + (l + t) * d, ki) > cpl_min) l += t;
    int j = i + l * d;
    int from = min(i, j), to = max(i, j);
    const Key kf = __ldg(codes + from);
    int cpl_node = cpl(codes, n, from, to, kf);
    int s = 0;
    for (int t = (l + 1) / 2; t >= 1; t = (t + 1) / 2) {
        if (cpl(codes, n, from, from + s + t, kf) > cpl_node) s += t;
        if (t <= 1) break;
    }
    int mid = from + s;
    left = (from == mid) ? mid + n - 1 : mid;
    right = (to == mid + 1) ? mid + 1 + n - 1 : mid + 1;
    left_size = mid - from + 1;
    right_size = to - mid;
}

template <typename Key>
__global__ void __launch_bounds__(256)
k_karras(const Key *__restrict__ codes, const uint32_t *__restrict__ ids, uint32_t n,
         NodeRec *__restrict__ nodes, uint32_t *__restrict__ parents, uint32_t *__restrict__ counters,
         const float *__restrict__ tris_in, TriRec *__restrict__ tris, float *__restrict__ tris_out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i + 1 < n) {
        int l, r, ls, rs;
        karras_split(codes, (int)n, (int)i, l, r, ls, rs);
        const uint32_t inner = n - 1;
        uint32_t llink = (uint32_t)l < inner ? (uint32_t)l : make_leaf((uint32_t)l - inner, 1u);
        uint32_t rlink = (uint32_t)r < inner ? (uint32_t)r : make_leaf((uint32_t)r - inner, 1u);
        nodes[i].q3 = make_uint4(llink, rlink, (uint32_t)ls, (uint32_t)rs);
        parents[l] = (i << 1) | 0u;
        parents[r] = (i << 1) | 1u;
        counters[i] = 0u;
    }
    // invert_triangle_permutation_cuda (:557-578): gather into Morton order
    const uint32_t id = __ldg(ids + i);
    const float *src = tris_in + (size_t)id * kTriFloats;
    float a[3], b[3], c[3];
    load_positions(src, a, b, c);
    TriRec t;
    t.v0 = make_float4(a[0], a[1], a[2], __uint_as_float(1u));
    t.v1 = make_float4(b[0], b[1], b[2], __uint_as_float(id));
    t.v2 = make_float4(c[0], c[1], c[2], 0.0f);
    tris[i] = t;
    if (tris_out) {
        const float2 *s2 = reinterpret_cast<const float2 *>(src);
        float2 *d2 = reinterpret_cast<float2 *>(tris_out + (size_t)i * kTriFloats);
#pragma unroll
        for (int j = 0; j < kTriFloats / 2; ++j) d2[j] = __ldg(s2 + j);
    }
}

// ------------------------------------------------------------------------- //
// kernel: bottom-up refit                                                     //
// ------------------------------------------------------------------------- //
//
// One thread per leaf climbs towards the root; the second thread to arrive at
// a node (counted with atomicAdd, release/acquire through __threadfence)
// unions the two child boxes, applies the reference's collapse rule (both
// children leaves with equal Morton codes -> one multi-triangle leaf,
// :300-331) and continues.  A node's box is stored in its parent's record.

__device__ __forceinline__ void write_slot(NodeRec *nd, uint32_t side, const float lo[3],
                                           const float hi[3])
{
    float *f = reinterpret_cast<float *>(nd);
    const int o = side ? 6 : 0;
    f[o + 0] = lo[0]; f[o + 1] = hi[0];
    f[o + 2] = lo[1]; f[o + 3] = hi[1];
    f[o + 4] = lo[2]; f[o + 5] = hi[2];
}

__device__ __forceinline__ void read_slot_cg(const NodeRec *nd, uint32_t side, float lo[3], float hi[3])
{
    const float *f = reinterpret_cast<const float *>(nd);
    const int o = side ? 6 : 0;
    lo[0] = __ldcg(f + o + 0); hi[0] = __ldcg(f + o + 1);
    lo[1] = __ldcg(f + o + 2); hi[1] = __ldcg(f + o + 3);
    lo[2] = __ldcg(f + o + 4); hi[2] = __ldcg(f + o + 5);
}

__device__ __forceinline__ uint32_t leaf_count_cg(uint32_t link, const TriRec *tris)
{
    uint32_t f = leaf_count_field(link);
    if (f < 63u) return f + 1u;
    return __float_as_uint(__ldcg(&tris[leaf_first(link)].v0.w));
}

template <typename Key>
__global__ void __launch_bounds__(256)
k_refit(const Key *__restrict__ codes, uint32_t n, NodeRec *__restrict__ nodes,
        const uint32_t *__restrict__ parents, uint32_t *__restrict__ counters,
        TriRec *__restrict__ tris, RootRec *__restrict__ root, uint32_t *__restrict__ flags)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float lo[3], hi[3];
    {
        TriRec t = tris[j];
        const float a[3] = {t.v0.x, t.v0.y, t.v0.z};
        const float b[3] = {t.v1.x, t.v1.y, t.v1.z};
        const float c[3] = {t.v2.x, t.v2.y, t.v2.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = ref_min(ref_min(a[k], b[k]), c[k]);
            hi[k] = ref_max(ref_max(a[k], b[k]), c[k]);
        }
    }
    uint32_t link = make_leaf(j, 1u);   // link of the current node, as its parent stores it
    bool link_changed = false;
    Key code = codes[j];
    uint32_t cur = n - 1 + j;
    if (n == 1) {
        for (int k = 0; k < 3; ++k) { root->lo[k] = lo[k]; root->hi[k] = hi[k]; }
        root->link = link;
        return;
    }
    // a path to the root has at most 2 * (key bits + index bits) nodes
    for (uint32_t climb = 0;; ++climb) {
        if (climb > 256u) {
            atomicOr(flags, RTA_DEV_ITER_LIMIT);
            return;
        }
        const uint32_t pl = parents[cur];
        const uint32_t p = pl >> 1, side = pl & 1u;
        if (p >= n - 1) {
            atomicOr(flags, RTA_DEV_BAD_LINK);
            return;
        }
        NodeRec *nd = nodes + p;
        write_slot(nd, side, lo, hi);
        if (link_changed) reinterpret_cast<uint32_t *>(&nd->q3)[side] = link;
        __threadfence();
        if (atomicAdd(counters + p, 1u) == 0u) return;   // first arrival stops
        __threadfence();
        float slo[3], shi[3];
        read_slot_cg(nd, side ^ 1u, slo, shi);
        const uint32_t sib = __ldcg(reinterpret_cast<const uint32_t *>(&nd->q3) + (side ^ 1u));
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = ref_min(lo[k], slo[k]);
            hi[k] = ref_max(hi[k], shi[k]);
        }
        if ((is_leaf(sib) ? leaf_first(sib) : sib) >= n) {
            atomicOr(flags, RTA_DEV_BAD_LINK);
            return;
        }
        const Key sib_code = is_leaf(sib) ? codes[leaf_first(sib)] : codes[sib];
        link_changed = false;
        uint32_t plink = p;
        if (code == sib_code && is_leaf(link) && is_leaf(sib)) {
            const uint32_t f0 = leaf_first(link), f1 = leaf_first(sib);
            const uint32_t cnt = leaf_count_cg(link, tris) + leaf_count_cg(sib, tris);
            const uint32_t first = f0 < f1 ? f0 : f1;
            tris[first].v0.w = __uint_as_float(cnt);
            plink = make_leaf(first, cnt);
            link_changed = true;
        }
        link = plink;
        code = codes[p];
        cur = p;
        if (p == 0) {
            for (int k = 0; k < 3; ++k) { root->lo[k] = lo[k]; root->hi[k] = hi[k]; }
            root->link = link;
            return;
        }
    }
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
    if (k != 0 && (parents[k] >> 1) >= n - 1) {   // only a broken build gets here
        out[2 * k + 0] = make_float4(0.f, 0.f, 0.f, 0.f);
        out[2 * k + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (k == 0) {
        for (int a = 0; a < 3; ++a) { lo[a] = root->lo[a]; hi[a] = root->hi[a]; }
        link = root->link;
    } else {
        const uint32_t pl = parents[k];
        const NodeRec *nd = nodes + (pl >> 1);
        const float *f = reinterpret_cast<const float *>(nd);
        const int o = (pl & 1u) ? 6 : 0;
        lo[0] = f[o + 0]; hi[0] = f[o + 1];
        lo[1] = f[o + 2]; hi[1] = f[o + 3];
        lo[2] = f[o + 4]; hi[2] = f[o + 5];
        link = reinterpret_cast<const uint32_t *>(&nd->q3)[pl & 1u];
    }
    uint32_t w0, w1;
    if (k >= n - 1) {
        w0 = 1u << 1;           // original leaves keep (tris = k-(n-1), elems = 1)
        w1 = k - (n - 1);
    } else if (is_leaf(link)) {  // a collapsed inner node
        uint32_t f = leaf_count_field(link);
        uint32_t cnt = (f < 63u || leaf_first(link) >= n) ? f + 1u : __float_as_uint(tris[leaf_first(link)].v0.w);
        w0 = cnt << 1;
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
    uint32_t *counters = nullptr;
    TriRec *tris = nullptr;
    uint32_t *status = nullptr;
    uint32_t n = 0;   // last build
    int last_bits = 30;
    bool smem_set = false;
};

static int bounds_blocks(uint32_t n)
{
    int want = (int)((n + kBoundsThreads - 1) / kBoundsThreads);
    int cap = num_sms() * 8;
    return want < cap ? (want > 0 ? want : 1) : cap;
}

static void free_ctx(rta_lbvh_ctx *c)
{
    void *ptrs[] = {c->keys0, c->keys1, c->vals0, c->vals1, c->cent, c->partial, c->state,
                    c->scratch, c->nodes, c->root, c->parents, c->counters, c->tris, c->status};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    uint32_t cap = 0;
    *c = rta_lbvh_ctx();
    c->cap = cap;
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
    delete ctx;
    return RTA_OK;
}

int rta_lbvh_reserve(rta_lbvh_ctx *c, uint32_t n, int bits)
{
    if (!c || n == 0 || n > kMaxTriangles || (bits != 30 && bits != 63)) return RTA_ERR_INVALID;
    if (n <= c->cap && (bits == 30 || c->bits == 63)) return RTA_OK;
    free_ctx(c);
    const size_t ksz = bits == 63 ? 8 : 4;
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    const int passes = bits == 63 ? 8 : 4;
    c->scratch_bytes = sizeof(SortScratchHeader) + (size_t)passes * tiles * kRadix * 4;
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
    RTA_CUDA_TRY(cudaMalloc(&c->tris, (size_t)n * sizeof(TriRec)));
    RTA_CUDA_TRY(cudaMalloc(&c->status, 64));
    RTA_CUDA_TRY(cudaMemset(c->status, 0, 64));
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
    const int passes = bits == 63 ? 8 : 4;
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    SortScratchHeader *hdr = reinterpret_cast<SortScratchHeader *>(c->scratch);
    uint32_t *tstat = reinterpret_cast<uint32_t *>(c->scratch + sizeof(SortScratchHeader));
    const size_t used = sizeof(SortScratchHeader) + (size_t)passes * tiles * kRadix * 4;
    RTA_CUDA_TRY(cudaMemsetAsync(c->scratch, 0, used, s));

    const float *tin = static_cast<const float *>(tris);
    const int bb = bounds_blocks(n);
    k_bounds<<<bb, kBoundsThreads, 0, s>>>(tin, n, c->cent, c->partial, c->state, c->status,
                                           bits == 63 ? 2097152.0f : 1024.0f);
    if ((rc = check_launch("k_bounds"))) return rc;
    const int eb = (int)((n + 255) / 256);
    const int mb = eb < num_sms() * 8 ? eb : num_sms() * 8;
    const uint32_t gmask = bits == 63 ? 0x1fffffu : 0x3ffu;
    if (bits == 63)
        k_morton<uint64_t><<<mb, 256, 0, s>>>(c->cent, n, (uint64_t *)c->keys0, c->state, hdr,
                                              c->status, passes, gmask);
    else
        k_morton<uint32_t><<<mb, 256, 0, s>>>(c->cent, n, (uint32_t *)c->keys0, c->state, hdr,
                                              c->status, passes, gmask);
    if ((rc = check_launch("k_morton"))) return rc;

    const size_t smem = bits == 63 ? sizeof(SortSmem<uint64_t>) : sizeof(SortSmem<uint32_t>);
    if (!c->smem_set) {
        RTA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint32_t>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(SortSmem<uint32_t>)));
        RTA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint64_t>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(SortSmem<uint64_t>)));
        c->smem_set = true;
    }
    void *kin = c->keys0, *kout = c->keys1;
    uint32_t *vin = nullptr, *vout = c->vals0;
    for (int p = 0; p < passes; ++p) {
        uint32_t *ts = tstat + (size_t)p * tiles * kRadix;
        if (bits == 63)
            k_onesweep<uint64_t><<<tiles, kSortThreads, smem, s>>>(
                (const uint64_t *)kin, vin, (uint64_t *)kout, vout, n, p, hdr, ts, c->status);
        else
            k_onesweep<uint32_t><<<tiles, kSortThreads, smem, s>>>(
                (const uint32_t *)kin, vin, (uint32_t *)kout, vout, n, p, hdr, ts, c->status);
        if ((rc = check_launch("k_onesweep"))) return rc;
        std::swap(kin, kout);
        vin = vout;
        vout = (vout == c->vals0) ? c->vals1 : c->vals0;
    }
    // an even number of passes leaves the keys in keys0; the values in `vin`
    uint32_t *ids = vin;
    if (ids != c->vals0) std::swap(c->vals0, c->vals1);   // keep sorted ids in vals0
    if (bits == 63)
        k_karras<uint64_t><<<eb, 256, 0, s>>>((const uint64_t *)c->keys0, c->vals0, n, c->nodes,
                                              c->parents, c->counters, tin, c->tris,
                                              (float *)tris_out);
    else
        k_karras<uint32_t><<<eb, 256, 0, s>>>((const uint32_t *)c->keys0, c->vals0, n, c->nodes,
                                              c->parents, c->counters, tin, c->tris,
                                              (float *)tris_out);
    if ((rc = check_launch("k_karras"))) return rc;
    if (bits == 63)
        k_refit<uint64_t><<<eb, 256, 0, s>>>((const uint64_t *)c->keys0, n, c->nodes, c->parents,
                                             c->counters, c->tris, c->root, c->status);
    else
        k_refit<uint32_t><<<eb, 256, 0, s>>>((const uint32_t *)c->keys0, n, c->nodes, c->parents,
                                             c->counters, c->tris, c->root, c->status);
    if ((rc = check_launch("k_refit"))) return rc;
    c->n = n;
    c->last_bits = bits;
    return RTA_OK;
}

int rta_lbvh_get(const rta_lbvh_ctx *c, rta_lbvh *out)
{
    if (!c || !out || c->n == 0) return RTA_ERR_INVALID;
    out->nodes = c->nodes;
    out->root = c->root;
    out->tris = c->tris;
    out->index = c->vals0;
    out->codes = c->keys0;
    out->parents = c->parents;
    out->n = c->n;
    out->morton_bits = c->last_bits;
    out->status = c->status;
    return RTA_OK;
}

int rta_lbvh_status(const rta_lbvh *bvh, rta_stream_t stream, uint32_t *flags)
{
    if (!bvh || !flags) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    RTA_CUDA_TRY(cudaMemcpy(flags, bvh->status, 4, cudaMemcpyDeviceToHost));
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
