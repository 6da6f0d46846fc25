// lbvh.cuh -- device pieces of the LBVH build shared by the one-mesh builder
// (build.cu) and the batched multi-mesh builder (batch.cu): build constants,
// position loads, Morton helpers, the onesweep radix pass, Karras' split
// search, the per-node link writer and the refit over Morton ranges.
#pragma once

#include <utility>

#include "batch.cuh"
#include "common.cuh"

namespace rta {

// ------------------------------------------------------------------------- //
// build state                                                                //
// ------------------------------------------------------------------------- //

constexpr int kTriFloats = 26;         // cuda::simple_triangle = 104 bytes
constexpr int kBoundsThreads = 256;
// 8 warps of 16 keys: 512 threads of 8 or 16 keys and 1024 of 4 measured
// slower at 4M 63-bit (0.845, 0.856, 0.933 against 0.832 ms), 256 of 8 at 3
// or 4 blocks per SM too (0.895, 0.881 ms)
#ifndef RTA_SORT_THREADS
#define RTA_SORT_THREADS 256
#endif
constexpr int kSortThreads = RTA_SORT_THREADS;
#ifndef RTA_SORT_ITEMS
#define RTA_SORT_ITEMS 16
#endif
constexpr int kSortItems = RTA_SORT_ITEMS;   // keys per thread
// blocks per SM the onesweep kernel must fit in registers.  With the
// lane-mask ranking, 2 (no spills) measured faster than 3 (80 registers,
// spills): 1M 30-bit build 0.214 against 0.224 ms, 4M 63-bit 0.866 against
// 0.891 ms (the two timed in alternating order); 12, 24 or 32 keys per
// thread were not faster
#ifndef RTA_SORT_MIN_BLOCKS
#define RTA_SORT_MIN_BLOCKS 2
#endif
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per tile
constexpr int kMaxDigitBits = 11;
constexpr int kMaxRadix = 1 << kMaxDigitBits;
constexpr int kMaxPasses = 8;          // 63-bit keys at 8 bits per digit

struct BuildState {
    float lo[3], hi[3], scale[3];
    uint32_t done;                 // bounds last-block ticket (self-resetting)
};

// Zeroed by one memset before every build.  hist holds the global digit
// histogram of pass p at hist[p * radix], radix = 2^digit bits.
struct SortScratchHeader {
    uint32_t tile_ctr[kMaxPasses];
    uint32_t hist[kMaxPasses * kMaxRadix];
    uint32_t n_cross;        // refit: inner nodes whose range crosses a segment border
    uint32_t refit_ticket;   // refit: last-group ticket of the group tables
};

// radix passes for `key_bits` bits at `digit_bits` per pass
__host__ __device__ __forceinline__ int sort_passes(int key_bits, int digit_bits)
{
    return (key_bits + digit_bits - 1) / digit_bits;
}

// bytes of the header that one build uses (the memset covers only these)
__host__ __device__ __forceinline__ size_t sort_header_bytes(int passes, int digit_bits)
{
    return sizeof(uint32_t) * kMaxPasses + sizeof(uint32_t) * (size_t)passes * ((size_t)1 << digit_bits);
}

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

// ------------------------------------------------------------------------- //
// Morton helpers                                                             //
// ------------------------------------------------------------------------- //

// float -> unsigned as the reference's `uint x = f;` compiles on the GPU
// (cvt.rzi.u32.f32: truncation, NaN and negatives to 0, saturation)
__device__ __forceinline__ uint32_t f2u_rz_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return __float2uint_rz(v);
}

// bit k of the low 11 bits of v moves to bit 3k (in 32-bit words)
__device__ __forceinline__ uint32_t spread3_11(uint32_t v)
{
    v &= 0x7ffu;
    v = (v | (v << 16)) & 0xff0000ffu;
    v = (v | (v << 8)) & 0x0f00f00fu;
    v = (v | (v << 4)) & 0xc30c30c3u;
    v = (v | (v << 2)) & 0x49249249u;
    return v;
}

// bit k of the low 21 bits of v moves to bit 3k: bits 0..10 and 11..20 spread
// in 32-bit words (the upper part lands at bit 33)
__device__ __forceinline__ uint64_t spread3(uint32_t v)
{
    return (uint64_t)spread3_11(v) | ((uint64_t)spread3_11((v >> 11) & 0x3ffu) << 33);
}

// morton_codes2 (lbvh-kernels.cu:174-180): (center - min) * d, to unsigned,
// masked to the grid, interleaved x -> bit 0, y -> bit 1, z -> bit 2
__device__ __forceinline__ uint64_t morton_code(const float c[3], const float lo[3], const float d[3],
                                                uint32_t grid_mask, bool &wrapped)
{
    uint32_t x = f2u_rz_sat(__fmul_rn(__fsub_rn(c[0], lo[0]), d[0]));
    uint32_t y = f2u_rz_sat(__fmul_rn(__fsub_rn(c[1], lo[1]), d[1]));
    uint32_t z = f2u_rz_sat(__fmul_rn(__fsub_rn(c[2], lo[2]), d[2]));
    wrapped |= (x > grid_mask) | (y > grid_mask) | (z > grid_mask);
    return spread3(x & grid_mask) | (spread3(y & grid_mask) << 1) | (spread3(z & grid_mask) << 2);
}

// one key's digits of sort passes [0, passes) into shared histograms (pass
// p's at hist + p * 2^DBITS); the digit shifts are constants
template <int DBITS, typename Key>
__device__ __forceinline__ void hist_add(uint32_t *hist, Key key, int passes)
{
    constexpr uint32_t kMask = (1u << DBITS) - 1u;
#pragma unroll
    for (int p = 0; p < kMaxPasses; ++p)
        if (DBITS * p < 64 && p < passes)
            atomicAdd(&hist[(p << DBITS) + ((uint32_t)((uint64_t)key >> (DBITS * p)) & kMask)], 1u);
}

// ------------------------------------------------------------------------- //
// one onesweep LSD radix pass                                                 //
// ------------------------------------------------------------------------- //
//
// A tile of 4096 keys per block: warp-level stable ranking by lane masks
// (each lane ORs its bit into a shared word of its digit; the word then names
// the lanes with equal digits, whatever the digit width), per-warp digit
// counters in shared memory, decoupled
// look-back across tiles for the per-digit prefix (Merrill & Garland's
// single-pass scan as used by Adinets & Merrill's Onesweep), a shared-memory
// staging of the tile in digit order, and coalesced runs out to global
// memory.  BITS is the digit width (8 to 11): wider digits mean fewer
// passes but larger per-warp counters and more look-back work per tile.

template <typename Key, int BITS>
struct SortSmem {
    static constexpr int kRadix = 1 << BITS;
    uint32_t whist[kSortThreads / 32][kRadix];
    uint32_t digit_start[kRadix];
    uint32_t glob[kRadix];
    uint32_t scan_tmp[2 * (kSortThreads / 32)];
    uint32_t tile;
    // the ranking's lane masks are dead once the tile is ranked, the staging
    // area is live only afterwards: they share the space
    union {
        uint32_t match[kSortThreads / 32][kRadix];   // per warp and digit: lanes holding that digit
        struct {
            Key keys[kSortTile];
            uint32_t vals[kSortTile];
        } stage;
    } u;
};

// block-wide exclusive scans of two values per thread (256 threads) with
// one set of barriers; tmp holds 2 words per warp
__device__ __forceinline__ void block_excl_scan2(uint32_t a, uint32_t b, uint32_t *tmp, uint32_t &ea,
                                                 uint32_t &eb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = a, y = b;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, x, off);
        const uint32_t v = __shfl_up_sync(0xffffffffu, y, off);
        if (lane >= off) {
            x += u;
            y += v;
        }
    }
    if (lane == 31) {
        tmp[2 * w] = x;
        tmp[2 * w + 1] = y;
    }
    __syncthreads();
    if (w == 0) {
        uint32_t p = lane < kSortThreads / 32 ? tmp[2 * lane] : 0u;
        uint32_t q = lane < kSortThreads / 32 ? tmp[2 * lane + 1] : 0u;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, p, off);
            const uint32_t v = __shfl_up_sync(0xffffffffu, q, off);
            if (lane >= off) {
                p += u;
                q += v;
            }
        }
        if (lane < kSortThreads / 32) {
            tmp[2 * lane] = p;
            tmp[2 * lane + 1] = q;
        }
    }
    __syncthreads();
    ea = (w ? tmp[2 * (w - 1)] : 0u) + x - a;
    eb = (w ? tmp[2 * (w - 1) + 1] : 0u) + y - b;
    __syncthreads();
}

// The kernel and its launcher have internal linkage: build.cu and batch.cu
// each instantiate them, and each translation unit must launch (and set the
// shared-memory attribute of) its own module's kernel.
namespace {

// One pass over digit bits [shift, shift + BITS).  vin == nullptr means the
// values are the key positions (first pass).  hist is this pass's global
// digit histogram, tstat its tile status words ([tile][radix]).  When
// code_out is set, the pass also writes (uint32_t)key & code_mask of every
// key at its output position (the batched build's last pass writes the
// per-mesh Morton codes this way).
template <typename Key, int BITS>
__global__ void __launch_bounds__(kSortThreads, RTA_SORT_MIN_BLOCKS)
k_onesweep(const Key *__restrict__ kin, const uint32_t *__restrict__ vin, Key *__restrict__ kout,
           uint32_t *__restrict__ vout, uint32_t n, int shift, uint32_t *__restrict__ tile_ctr,
           const uint32_t *__restrict__ hist, uint32_t *__restrict__ tstat, uint32_t *__restrict__ flags,
           uint32_t *__restrict__ code_out, uint32_t code_mask)
{
    pdl_enter();
    constexpr int kRadix = 1 << BITS;
    constexpr uint32_t kDigitMask = (uint32_t)kRadix - 1u;
    constexpr int kDpt = kRadix > kSortThreads ? kRadix / kSortThreads : 1;   // digits per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem<Key, BITS> &S = *reinterpret_cast<SortSmem<Key, BITS> *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;

    if (tid == 0) S.tile = atomicAdd(tile_ctr, 1u);
    for (int j = tid; j < (kSortThreads / 32) * kRadix; j += kSortThreads) {
        (&S.whist[0][0])[j] = 0;
        (&S.u.match[0][0])[j] = 0;
    }
    __syncthreads();
    const uint32_t tile = S.tile;
    const uint32_t base = tile * kSortTile;
    const uint32_t wbase = base + (uint32_t)w * (32 * kSortItems);

    // this pass's global digit counts, loaded now and used after the ranking
    uint32_t gh[kDpt];
#pragma unroll
    for (int j = 0; j < kDpt; ++j) gh[j] = tid * kDpt + j < kRadix ? hist[tid * kDpt + j] : 0u;

    // (Keeping only the digits in registers through the ranking and loading
    // keys and values again for the staging, 80 registers and three blocks
    // per SM, measured no faster: the second load's latency ate the gain.)
    Key k[kSortItems];
    uint32_t v[kSortItems];
    uint32_t rank[kSortItems];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = wbase + i * 32 + lane;
        bool ok = idx < n;
        k[i] = ok ? kin[idx] : (Key)~(Key)0;
        v[i] = ok ? (vin ? vin[idx] : idx) : 0u;
    }
    auto digit = [&](int i) -> uint32_t { return (uint32_t)(k[i] >> shift) & kDigitMask; };
    // Stable rank of each key among the warp's keys of its digit, in (item,
    // lane) order: the lanes OR their bit into the digit's mask word; the
    // highest lane of a mask is its leader, adds the lane count to the warp's
    // digit counter and clears the word; the others take the old counter
    // from it.  The warp's keys are consecutive in the input (item-major),
    // so the order is the input order.  (Ranking two items at a time, two
    // independent chains, measured no faster.)
    const uint32_t lane_bit = 1u << lane;
    const uint32_t le_mask = lane_bit | (lane_bit - 1u);
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t d = digit(i);
        uint32_t *m = &S.u.match[w][d];
        atomicOr(m, lane_bit);
        __syncwarp();
        const uint32_t peers = *m;
        const int leader = 31 - __clz(peers);
        const uint32_t upto = __popc(peers & le_mask);   // 1-based position among the peers
        uint32_t off = 0;
        if (lane == leader) off = atomicAdd(&S.whist[w][d], upto);   // the leader's upto = all peers
        off = __shfl_sync(0xffffffffu, off, leader);
        __syncwarp();   // every lane has read the mask
        if (lane == leader) *m = 0u;
        __syncwarp();
        rank[i] = off + upto - 1u;
    }
    __syncthreads();

    // per digit (thread tid owns digits tid*kDpt .. tid*kDpt+kDpt-1): warp
    // offsets, tile count, block offsets
    uint32_t cnt[kDpt];
    uint32_t csum = 0, gsum = 0;
    // padding keys (beyond n) are all the last digit and sit at the end of the last tile
    const uint32_t valid = n - base < (uint32_t)kSortTile ? n - base : (uint32_t)kSortTile;
    const uint32_t pad = (uint32_t)kSortTile - valid;
#pragma unroll
    for (int j = 0; j < kDpt; ++j) {
        const int d = tid * kDpt + j;
        cnt[j] = 0;
        if (d < kRadix) {
#pragma unroll
            for (int q = 0; q < kSortThreads / 32; ++q) {
                uint32_t c = S.whist[q][d];
                S.whist[q][d] = cnt[j];
                cnt[j] += c;
            }
            const uint32_t cv = (d == kRadix - 1) ? cnt[j] - pad : cnt[j];
            uint32_t *my_stat = tstat + (size_t)tile * kRadix + d;
            st_volatile(my_stat, (tile == 0 ? kStatPrefix : kStatAggregate) | cv);
        }
        csum += cnt[j];
        gsum += gh[j];
    }
    uint32_t start0, gexcl0;
    block_excl_scan2(csum, gsum, S.scan_tmp, start0, gexcl0);
    uint32_t dstart[kDpt];
    {
        uint32_t start = start0;
#pragma unroll
        for (int j = 0; j < kDpt; ++j) {
            const int d = tid * kDpt + j;
            dstart[j] = start;
            if (d < kRadix) S.digit_start[d] = start;
            start += cnt[j];
        }
    }
    __syncthreads();

    // the tile in digit order in shared memory; meanwhile the predecessor
    // tiles get further with their prefixes
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t d = digit(i);
        rank[i] += S.digit_start[d] + S.whist[w][d];
    }
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        S.u.stage.keys[rank[i]] = k[i];
        S.u.stage.vals[rank[i]] = v[i];
    }
    {
        uint32_t gexcl = gexcl0;
#pragma unroll
        for (int j = 0; j < kDpt; ++j) {
            const int d = tid * kDpt + j;
            if (d < kRadix) {
                const uint32_t cv = (d == kRadix - 1) ? cnt[j] - pad : cnt[j];
                uint32_t excl = 0;
                if (tile > 0) {
                    // a status word carries its flag and its count in one
                    // 32-bit store and nothing else is read on its account,
                    // so no fence orders it against other memory
                    excl = lookback(tstat + d, kRadix, tile, flags);
                    st_volatile(tstat + (size_t)tile * kRadix + d, kStatPrefix | ((excl + cv) & kStatValue));
                }
                S.glob[d] = gexcl + excl - dstart[j];
            }
            gexcl += gh[j];
        }
    }
    __syncthreads();
    if (valid == (uint32_t)kSortTile) {   // every tile but the last: a fixed trip count, unrolled
#pragma unroll
        for (int r = 0; r < kSortItems; ++r) {
            const uint32_t j = (uint32_t)tid + (uint32_t)r * kSortThreads;
            const Key key = S.u.stage.keys[j];
            const uint32_t dst = S.glob[(uint32_t)(key >> shift) & kDigitMask] + j;
            kout[dst] = key;
            vout[dst] = S.u.stage.vals[j];
            if (code_out) code_out[dst] = (uint32_t)key & code_mask;
        }
    } else {
        for (uint32_t j = tid; j < valid; j += kSortThreads) {
            const Key key = S.u.stage.keys[j];
            const uint32_t dst = S.glob[(uint32_t)(key >> shift) & kDigitMask] + j;
            kout[dst] = key;
            vout[dst] = S.u.stage.vals[j];
            if (code_out) code_out[dst] = (uint32_t)key & code_mask;
        }
    }
}

// Launches the P passes of one LSD sort of n keys with BITS-bit digits.  The
// header's tile counters and histograms (filled by the Morton kernel) and the
// tile status words are zero on entry.  On return *keys_sorted / *vals_sorted
// point at the buffers holding the result (ping-pong between the two pairs).
template <typename Key, int BITS>
int sort_passes_launch(Key *k0, Key *k1, uint32_t *v0, uint32_t *v1, uint32_t n, int passes,
                       SortScratchHeader *hdr, uint32_t *tstat, uint32_t *flags, uint32_t *code_out,
                       uint32_t code_mask, cudaStream_t s, Key **keys_sorted, uint32_t **vals_sorted,
                       bool pdl = false)
{
    constexpr int kRadix = 1 << BITS;
    static bool smem_set = false;
    const size_t smem = sizeof(SortSmem<Key, BITS>);
    if (!smem_set) {
        RTA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<Key, BITS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        smem_set = true;
    }
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    Key *kin = k0, *kout = k1;
    uint32_t *vin = nullptr, *vout = v0;
    for (int p = 0; p < passes; ++p) {
        uint32_t *ts = tstat + (size_t)p * tiles * kRadix;
        const cudaError_t e =
            launch_pdl(pdl, k_onesweep<Key, BITS>, dim3(tiles), dim3(kSortThreads), smem, s, kin,
                       (const uint32_t *)vin, kout, vout, n, BITS * p, hdr->tile_ctr + p,
                       (const uint32_t *)(hdr->hist + (size_t)p * kRadix), ts, flags,
                       p == passes - 1 ? code_out : nullptr, code_mask);
        if (e != cudaSuccess) {
            set_cuda_error(e, "k_onesweep");
            return RTA_ERR_CUDA;
        }
        std::swap(kin, kout);
        vin = vout;
        vout = (vout == v0) ? v1 : v0;
    }
    *keys_sorted = kin;
    *vals_sorted = vin;
    return RTA_OK;
}

} // namespace

// The refit works on segments of 256 consecutive leaves; 128 measured slower
// (more nodes cross segments: 1M build 0.270 against 0.261 ms)
#ifndef RTA_REFIT_SEG_LOG2
#define RTA_REFIT_SEG_LOG2 8
#endif
constexpr uint32_t kRefitSeg = 1u << RTA_REFIT_SEG_LOG2;   // leaves per segment = threads per block
constexpr int kRefitLevels = RTA_REFIT_SEG_LOG2;           // sparse table levels (windows of 1 .. kRefitSeg / 2)

__device__ __forceinline__ bool crosses_segment(uint32_t gl, uint32_t gr) { return gl / kRefitSeg != gr / kRefitSeg; }

// A parent word is (parent << 1) | side, with kParentCrosses set when the
// parent's Morton range crosses a segment border (the refit's bookkeeping).
constexpr uint32_t kParentCrosses = 1u << 31;
// A link record's size words (z, w) carry kCollapses when that child is an
// inner node whose codes are all equal (it becomes a leaf of the parent).
constexpr uint32_t kCollapses = 1u << 31;
__device__ __forceinline__ uint32_t parent_index(uint32_t pl) { return (pl & ~kParentCrosses) >> 1; }

// ------------------------------------------------------------------------- //
// Karras radix tree                                                           //
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
// (clz of a zero key difference is the key width, which is the tie-break's
// base, so equal codes need no branch)
template <typename Key>
__device__ __forceinline__ int cpl(const Key *__restrict__ codes, int n, int i, int j, Key ki)
{
    if ((unsigned)j >= (unsigned)n) return -1;
    const Key x = ki ^ __ldg(codes + j);
    const int c = KeyBits<Key>::clz(x);
    return x == 0 ? c + __clz(i ^ j) : c;
}

// The searches below only ask whether cpl(base, j) > c for a fixed c: with
// x = codes[base] ^ codes[j], that is x < 2^(W-1-c) for c < W (key width W,
// equal codes included), x == 0 and base ^ j < 2^(W+31-c) for c >= W (the
// index tie-break), and true for c = -1 (codes use at most W - 1 bits) --
// a compare instead of the leading-zero counts.
template <typename Key>
__device__ __forceinline__ void prefix_threshold(int c, Key &th, uint32_t &tl)
{
    constexpr int W = KeyBits<Key>::tie;
    if (c < 0) {
        th = ~(Key)0;
        tl = 0u;
    } else if (c < W) {
        th = (Key)1 << (W - 1 - c);
        tl = 0u;
    } else {
        th = 0;
        tl = 1u << (W + 31 - c);
    }
}

// cpl(base, j) > c, c given by its threshold (th, tl); false out of range
template <typename Key>
__device__ __forceinline__ bool longer_prefix(const Key *__restrict__ codes, int n, int base, int j, Key kb, Key th,
                                              uint32_t tl)
{
    if ((unsigned)j >= (unsigned)n) return false;
    const Key x = kb ^ __ldg(codes + j);
    return x < th || (x == th && (uint32_t)(base ^ j) < tl);
}

// (Leaving the nodes whose range search passes 64 leaves to a second launch,
// so that one warp's searches have alike trip counts, measured no faster:
// the serialised passes went 29 -> 41 us at 1M and 105 -> 112 us at 4M.)
template <typename Key>
__device__ __forceinline__ void karras_split(const Key *__restrict__ codes, int n, int i, int &left,
                                             int &right, int &left_size, int &right_size)
{
    // build_tree_karras (:205-249): direction, range end (exponential +
    // binary search), split (binary search with ceiling halving)
    const Key ki = __ldg(codes + i);
    const int c_next = cpl(codes, n, i, i + 1, ki), c_prev = cpl(codes, n, i, i - 1, ki);
    const int d = c_next - c_prev >= 0 ? 1 : -1;
    Key th;
    uint32_t tl;
    prefix_threshold(d > 0 ? c_prev : c_next, th, tl);   // cpl_min = cpl(i, i - d)
    int l_max = 2;
    while (longer_prefix(codes, n, i, i + l_max * d, ki, th, tl)) l_max *= 2;
    int l = 0;
    for (int t = l_max / 2; t >= 1; t /= 2)
        if (longer_prefix(codes, n, i, i + (l + t) * d, ki, th, tl)) l += t;
    int j = i + l * d;
    int from = min(i, j), to = max(i, j);
    const Key kf = __ldg(codes + from);
    prefix_threshold(cpl(codes, n, from, to, kf), th, tl);   // cpl_node
    int s = 0;
    for (int t = (l + 1) / 2; t >= 1; t = (t + 1) / 2) {
        if (longer_prefix(codes, n, from, from + s + t, kf, th, tl)) s += t;
        if (t <= 1) break;
    }
    int mid = from + s;
    left = (from == mid) ? mid + n - 1 : mid;
    right = (to == mid + 1) ? mid + 1 + n - 1 : mid + 1;
    left_size = mid - from + 1;
    right_size = to - mid;
}

// links of inner node i (i + 1 < n) of a tree over codes[0, n) -- (left
// link, right link, left size, right size), into a compact array the refit
// reads; the refit writes each node's whole record -- and its children's
// parent words, flagged when node i's range crosses a segment border (the
// tree's leaves start at leaf position base of the segmented sequence)
template <typename Key>
__device__ __forceinline__ void karras_node(const Key *__restrict__ codes, uint32_t n, uint32_t i,
                                            uint4 *__restrict__ links, uint32_t *__restrict__ parents,
                                            uint32_t base = 0u)
{
    int l, r, ls, rs;
    karras_split(codes, (int)n, (int)i, l, r, ls, rs);
    const uint32_t inner = n - 1;
    uint32_t llink = (uint32_t)l < inner ? (uint32_t)l : make_leaf((uint32_t)l - inner, 1u);
    uint32_t rlink = (uint32_t)r < inner ? (uint32_t)r : make_leaf((uint32_t)r - inner, 1u);
    const uint32_t mid = (uint32_t)l < inner ? (uint32_t)l : (uint32_t)l - inner;   // the split
    // an inner child whose codes are all equal collapses to a leaf: flagged
    // in its size word for the refit
    const uint32_t from = mid + 1u - (uint32_t)ls, to = mid + (uint32_t)rs;
    const bool lcol = ls > 1 && __ldg(codes + from) == __ldg(codes + mid);
    const bool rcol = rs > 1 && __ldg(codes + mid + 1u) == __ldg(codes + to);
    links[i] = make_uint4(llink, rlink, (uint32_t)ls | (lcol ? kCollapses : 0u), (uint32_t)rs | (rcol ? kCollapses : 0u));
    const uint32_t cross = crosses_segment(base + from, base + to) ? kParentCrosses : 0u;
    parents[l] = (i << 1) | 0u | cross;
    parents[r] = (i << 1) | 1u | cross;
}

// The Morton-ordered 48-byte triangles are gathered in the Karras kernels,
// whose split searches are latency-bound and leave the memory system idle;
// the refit then reads them in order.  Measured against gathering them in
// k_refit_seg: 4M 63-bit build 0.791 -> 0.778 ms, 1M 30-bit level.
#ifndef RTA_KARRAS_GATHER
#define RTA_KARRAS_GATHER 1
#endif

// the Morton-ordered record of one triangle (count 1 until the refit
// collapses leaves; id = the triangle's index in its mesh's input)
__device__ __forceinline__ TriRec make_tri(const float *__restrict__ src, uint32_t id)
{
    float a[3], b[3], c[3];
    load_positions(src, a, b, c);
    TriRec t;
    t.v0 = make_float4(a[0], a[1], a[2], __uint_as_float(1u));
    t.v1 = make_float4(b[0], b[1], b[2], __uint_as_float(id));
    t.v2 = make_float4(c[0], c[1], c[2], 0.0f);
    return t;
}

// ------------------------------------------------------------------------- //
// refit over Morton ranges                                                    //
// ------------------------------------------------------------------------- //
//
// A node's box is the union of the leaf boxes over its Morton range [l, r],
// so every node's box is a range query over the sorted leaves: no climb, no
// arrival counters, no chain of dependent memory accesses.  The union is the
// reference's (lbvh-kernels.cu:305-312) with the right child arriving
// second: min = R < L ? R : L, max = R > L ? R : L, i.e. of equal values the
// left one is kept.  Over a range that keeps the leftmost leaf among those
// attaining the min (max) -- an associative rule, so any split of the range
// (overlapping windows included) gives the bits of the CPU restatement's
// sequential climb.  (Only NaN coordinates make the result depend on the
// grouping; the reference GPU climb is arrival-order dependent there.)
//
// The equal-code collapse (:300-331) makes a node a leaf exactly when all
// codes of its range are equal (codes[l] == codes[r], the codes are sorted):
// its link in the parent record becomes (first l, count r - l + 1), and the
// triangle record at l keeps the count of the largest collapsed node that
// starts there (atomic max; a climb writes the counts bottom-up).
//
// Node records are written whole where possible: an inner node whose range
// lies in one segment takes both children's boxes from the segment's table
// and writes its 64-byte record (boxes and links, collapsed children as
// leaf links) in one piece.  Only the children of a node whose range crosses
// a segment border write their box into its record slot by slot (a few per
// cent of the nodes); k_refit_ext writes such a node's links.
//
// The leaves of all meshes of a batch are one sorted sequence (a mesh's
// leaves are contiguous), and a node's range never leaves its mesh, so the
// segment tables below are built across mesh borders and the queries stay
// exact.  Three launches:
//   k_refit_seg  one block per 256-leaf segment: a shared-memory sparse table
//                of the leaf boxes; writes the record of each inner node
//                whose range lies in the segment (a mesh's root also into its
//                root record), the box of each leaf and such node whose
//                parent crosses a border into that parent's record, the
//                segment union, and lists the inner nodes whose range crosses
//                a segment border, each with the union of its range's part in
//                this segment (a suffix at l or a prefix at r);
//   k_refit_top  the same tables over the segment unions in 256-entry groups,
//                and in the last block a full sparse table over the groups;
//   k_refit_ext  each listed node: its links, and its box = suffix of its
//                first segment + segment unions between + prefix of its last
//                segment, into its parent's record (or the root record).

__device__ __forceinline__ void write_slot(NodeRec *nd, uint32_t side, const float lo[3],
                                           const float hi[3])
{
    float *f = reinterpret_cast<float *>(nd);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f[slot_lo(side, k)] = lo[k];
        f[slot_hi(side, k)] = hi[k];
    }
}

// group unions whose full table k_refit_top builds in shared memory (two
// levels in the segment table's space); more go level by level through L2
constexpr uint32_t kMaxGroups = kRefitLevels * kRefitSeg / 2;

struct Box6 {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box6 box_join(const Box6 &L, const Box6 &R)
{
    Box6 o;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.lo[k] = ref_min(R.lo[k], L.lo[k]);
        o.hi[k] = ref_max(R.hi[k], L.hi[k]);
    }
    return o;
}

__device__ __forceinline__ Box6 leaf_box(const TriRec &t)
{
    const float a[3] = {t.v0.x, t.v0.y, t.v0.z}, b[3] = {t.v1.x, t.v1.y, t.v1.z}, c[3] = {t.v2.x, t.v2.y, t.v2.z};
    Box6 o;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.lo[k] = ref_min(ref_min(a[k], b[k]), c[k]);
        o.hi[k] = ref_max(ref_max(a[k], b[k]), c[k]);
    }
    return o;
}

// boxes in global memory: 24 bytes, (lo.x, lo.y) (lo.z, hi.x) (hi.y, hi.z)
__device__ __forceinline__ Box6 gload(const float *base, size_t i)
{
    const float2 *p = reinterpret_cast<const float2 *>(base + 6 * i);
    const float2 a = p[0], b = p[1], c = p[2];
    return Box6{{a.x, a.y, b.x}, {b.y, c.x, c.y}};
}
__device__ __forceinline__ Box6 gload_cg(const float *base, size_t i)
{
    const float2 *p = reinterpret_cast<const float2 *>(base + 6 * i);
    const float2 a = __ldcg(p), b = __ldcg(p + 1), c = __ldcg(p + 2);
    return Box6{{a.x, a.y, b.x}, {b.y, c.x, c.y}};
}
__device__ __forceinline__ void gstore(float *base, size_t i, const Box6 &x)
{
    float2 *p = reinterpret_cast<float2 *>(base + 6 * i);
    p[0] = make_float2(x.lo[0], x.lo[1]);
    p[1] = make_float2(x.lo[2], x.hi[0]);
    p[2] = make_float2(x.hi[1], x.hi[2]);
}

__device__ __forceinline__ int floor_log2(uint32_t v) { return 31 - __clz(v); }

// The leaf tables of k_refit_seg keep levels 0 .. kSegLevels - 1 (windows
// up to 16 leaves, 30 KB); a longer range joins several top windows.  Six
// blocks per SM (40 registers) leave 60 KB of L1 for the gathers.  Measured
// against all 8 levels at 4 blocks (48 KB): 1M 30-bit build 0.203 -> 0.197
// ms, 4M 63-bit 0.832 -> 0.802 ms.  Tables of 6 or 7 levels at 6 or 5 blocks
// (over 200 KB of shared memory, 28 KB of L1) measured 0.91-0.93 ms; 4 levels
// at 6 blocks 0.807 ms; 5 or 4 levels at 7 blocks spill (0.95 ms).
#ifndef RTA_REFIT_SEG_LEVELS
#define RTA_REFIT_SEG_LEVELS 5
#endif
constexpr int kSegLevels = RTA_REFIT_SEG_LEVELS;
#ifndef RTA_REFIT_MIN_BLOCKS
#define RTA_REFIT_MIN_BLOCKS 6
#endif

// the sparse table of one segment in shared memory: level k, axis c,
// entry i; LEVELS levels (windows of 1 .. 2^(LEVELS - 1) entries)
template <int LEVELS>
struct SegTable {
    float2 (*t)[3][kRefitSeg];   // per level and axis: (lo, hi) of entry i
    __device__ __forceinline__ Box6 get(int k, uint32_t i) const
    {
        const float2 x = t[k][0][i], y = t[k][1][i], z = t[k][2][i];
        return Box6{{x.x, y.x, z.x}, {x.y, y.y, z.y}};
    }
    __device__ __forceinline__ void put(int k, uint32_t i, const Box6 &b)
    {
        t[k][0][i] = make_float2(b.lo[0], b.hi[0]);
        t[k][1][i] = make_float2(b.lo[1], b.hi[1]);
        t[k][2][i] = make_float2(b.lo[2], b.hi[2]);
    }
    // union over entries [a, b] of the segment: two overlapping windows, or
    // top windows from a on and one ending at b (joined left to right)
    __device__ __forceinline__ Box6 query(uint32_t a, uint32_t b) const
    {
        const uint32_t len = b - a + 1u;
        if (LEVELS >= kRefitLevels || len <= (2u << (LEVELS - 1))) {
            const int k = min(floor_log2(len), LEVELS - 1);
            return box_join(get(k, a), get(k, b + 1u - (1u << k)));
        }
        constexpr uint32_t W = 1u << (LEVELS - 1);
        Box6 x = get(LEVELS - 1, a);
        for (uint32_t s = a + W; s + W - 1u < b; s += W) x = box_join(x, get(LEVELS - 1, s));
        return box_join(x, get(LEVELS - 1, b + 1u - W));
    }
    // level 0 holds one box per thread; each level's entry joins the thread's
    // own entry of the level below (kept in registers) with the one half a
    // window further on
    __device__ __forceinline__ void build(const Box6 &x)
    {
        const uint32_t t_ = threadIdx.x;
        Box6 y = x;
        put(0, t_, y);
        __syncthreads();
#pragma unroll 1
        for (int k = 1; k < LEVELS; ++k) {
            const uint32_t half = 1u << (k - 1);
            if (t_ + half < kRefitSeg) y = box_join(y, get(k - 1, t_ + half));
            put(k, t_, y);
            __syncthreads();
        }
    }
};

__device__ __forceinline__ Box6 t1_query(const float *t1, uint32_t nseg, uint32_t a, uint32_t b)
{
    const int k = min(floor_log2(b - a + 1u), kRefitLevels - 1);
    const float *lv = t1 + 6 * (size_t)k * nseg;
    return box_join(gload(lv, a), gload(lv, b + 1u - (1u << k)));
}

// Morton range [l, r] (local to its mesh) of an inner node from its record:
// the right child's index, or its leaf's (or collapsed leaf's) first
// triangle, is split + 1 whichever of the three the record holds, and the
// subtree sizes give the ends.
__device__ __forceinline__ bool node_range(const uint4 q3, uint32_t n, uint32_t &l, uint32_t &r)
{
    const uint32_t rf = is_leaf(q3.y) ? leaf_first(q3.y) : q3.y;   // split + 1
    const uint32_t ls = q3.z & ~kCollapses, rs = q3.w & ~kCollapses;
    if (rf == 0u || ls == 0u || rs == 0u || ls > rf || rs > n - rf) return false;
    l = rf - ls;
    r = rf + rs - 1u;
    return true;
}

// The mesh that leaf position j (global) belongs to.  One tree: the whole
// range.  A batch: the mesh id is the sorted key's top bits.
struct MeshSpan {
    uint32_t m, tri_off, n, node_off, parent_off;
};
template <bool BATCH>
__device__ __forceinline__ MeshSpan mesh_of(uint32_t j, uint32_t n_all, const MeshRec *__restrict__ meshes,
                                            const uint64_t *__restrict__ keys)
{
    if (!BATCH) return MeshSpan{0u, 0u, n_all, 0u, 0u};
    const uint32_t m = (uint32_t)(keys[j] >> 30);
    const MeshRec mr = meshes[m];
    return MeshSpan{m, mr.tri_off, mr.n_tris, mr.node_off, mr.parent_off};
}

// whether the parent (word pl) of a node of mesh sp has a range that crosses
// a segment border; false with the bad-link flag for an index out of range
__device__ __forceinline__ bool parent_crosses(uint32_t pl, const MeshSpan &sp, uint32_t *__restrict__ flags)
{
    if (parent_index(pl) >= sp.n - 1u) {
        atomicOr(flags, RTA_DEV_BAD_LINK);
        return false;
    }
    return (pl & kParentCrosses) != 0u;
}

// a child's link in its parent's record: an inner child whose codes are all
// equal collapses to a leaf of its gr - gl + 1 triangles (the triangle record
// at gl keeps the largest such count)
// (the Karras kernel flagged that case in the child's size word)
__device__ __forceinline__ uint32_t child_link(uint32_t size_word, const MeshSpan &sp, uint32_t link, uint32_t gl,
                                               uint32_t gr, TriRec *__restrict__ tris)
{
    if (is_leaf(link) || !(size_word & kCollapses)) return link;
    const uint32_t cnt = gr - gl + 1u;
    atomicMax(reinterpret_cast<uint32_t *>(&tris[gl].v0.w), cnt);
    return make_leaf(gl - sp.tri_off, cnt);
}

// a mesh's root record: box, and a leaf link if all its codes are equal
template <typename Key>
__device__ __forceinline__ void write_root(const Key *__restrict__ codes, const MeshSpan &sp, const Box6 &x,
                                           TriRec *__restrict__ tris, RootRec *__restrict__ roots)
{
    const uint32_t gl = sp.tri_off, gr = sp.tri_off + sp.n - 1u;
    const bool collapsed = codes[gl] == codes[gr];
    if (collapsed) atomicMax(reinterpret_cast<uint32_t *>(&tris[gl].v0.w), sp.n);
    RootRec &R = roots[sp.m];
    for (int a = 0; a < 3; ++a) {
        R.lo[a] = x.lo[a];
        R.hi[a] = x.hi[a];
    }
    R.link = collapsed ? make_leaf(0u, sp.n) : 0u;
}

// a whole inner-node record: both children's boxes, planes interleaved as
// (left, right, left, right) per axis, and the links
__device__ __forceinline__ void write_record(NodeRec *nd, const Box6 &L, const Box6 &R, const uint4 q3)
{
    nd->q0 = make_float4(L.lo[0], R.lo[0], L.hi[0], R.hi[0]);
    nd->q1 = make_float4(L.lo[1], R.lo[1], L.hi[1], R.hi[1]);
    nd->q2 = make_float4(L.lo[2], R.lo[2], L.hi[2], R.hi[2]);
    nd->q3 = q3;
}

namespace {

template <typename Key, bool BATCH>
__global__ void __launch_bounds__(kRefitSeg, RTA_REFIT_MIN_BLOCKS)
k_refit_seg(const Key *__restrict__ codes, uint32_t n_all, const MeshRec *__restrict__ meshes,
            const uint64_t *__restrict__ keys, const float *__restrict__ tris_in, uint32_t *__restrict__ ids,
            NodeRec *__restrict__ nodes, const uint4 *__restrict__ links, const uint32_t *__restrict__ parents,
            TriRec *__restrict__ tris, RootRec *__restrict__ roots, float *__restrict__ pre,
            float *__restrict__ suf, float *__restrict__ seg, uint32_t *__restrict__ cross,
            uint32_t *__restrict__ n_cross, uint32_t *__restrict__ flags)
{
    pdl_enter();
    __shared__ float2 s_t[kSegLevels][3][kRefitSeg];
    SegTable<kSegLevels> T{s_t};
    const uint32_t t = threadIdx.x, base = blockIdx.x * kRefitSeg, j = base + t;
    const uint32_t cnt = min(kRefitSeg, n_all - base);
    Box6 b{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    // this thread's loads are issued before the table build and land meanwhile
    MeshSpan sp{0u, 0u, 1u, 0u, 0u};
    uint32_t leaf_pl = 0u, node_pl = 0u, jl = 0u;
    uint4 q3 = make_uint4(0u, 0u, 0u, 0u);
    if (j < n_all) {
        sp = mesh_of<BATCH>(j, n_all, meshes, keys);
        jl = j - sp.tri_off;
        if (sp.n > 1u) leaf_pl = parents[sp.parent_off + sp.n - 1u + jl];
        if (jl + 1u < sp.n) {
            q3 = links[sp.node_off + jl];
            if (jl != 0u) node_pl = parents[sp.parent_off + jl];
        }
        // invert_triangle_permutation_cuda (lbvh-kernels.cu:557-578): the
        // triangle of sorted position j, in Morton order, with its id local
        // to its mesh (collapse counts land in .w after the table build's
        // barrier, or in a later kernel)
        TriRec tr;
        if (tris_in) {
            const uint32_t id = ids[j], lid = id - sp.tri_off;
            tr = make_tri(tris_in + (size_t)id * kTriFloats, lid);
            tris[j] = tr;
            if (BATCH) ids[j] = lid;
        } else {   // gathered by the Karras kernel
            tr = tris[j];
        }
        b = leaf_box(tr);
    }
    T.build(b);
    bool crosses = false;
    if (j < n_all) {
        if (t == 0u) gstore(seg, blockIdx.x, T.query(0u, cnt - 1u));
        // the mesh's last leaf: the prefix a crossing node ending there reads
        if (jl + 1u == sp.n && sp.n > 1u) gstore(pre, j, T.query(0u, t));
        if (sp.n == 1u) {   // a one-triangle mesh: its root is the leaf
            RootRec &R = roots[sp.m];
            for (int a = 0; a < 3; ++a) {
                R.lo[a] = b.lo[a];
                R.hi[a] = b.hi[a];
            }
            R.link = make_leaf(0u, 1u);
        } else if (parent_crosses(leaf_pl, sp, flags)) {
            // the leaf's box into its parent's record (a parent within one
            // segment writes its record itself)
            write_slot(nodes + sp.node_off + parent_index(leaf_pl), leaf_pl & 1u, b.lo, b.hi);
        }
        // inner node jl of the mesh (one end of its range): its record here
        // when the range lies in this segment, else on the list for k_refit_ext
        uint32_t l, r;
        if (jl + 1u < sp.n) {
            if (!node_range(q3, sp.n, l, r)) {
                atomicOr(flags, RTA_DEV_BAD_LINK);
            } else {
                const uint32_t gl = sp.tri_off + l, gr = sp.tri_off + r, gm = gr + 1u - (q3.w & ~kCollapses);   // gm: right child's first
                if (!crosses_segment(gl, gr)) {
                    const Box6 bl = T.query(gl - base, gm - 1u - base), br = T.query(gm - base, gr - base);
                    const uint4 q = make_uint4(child_link(q3.z, sp, q3.x, gl, gm - 1u, tris),
                                               child_link(q3.w, sp, q3.y, gm, gr, tris), q3.z & ~kCollapses,
                                               q3.w & ~kCollapses);
                    write_record(nodes + sp.node_off + jl, bl, br, q);
                    if (jl == 0u) {
                        write_root(codes, sp, box_join(bl, br), tris, roots);
                    } else if (parent_crosses(node_pl, sp, flags)) {
                        const Box6 x = box_join(bl, br);
                        write_slot(nodes + sp.node_off + parent_index(node_pl), node_pl & 1u, x.lo, x.hi);
                    }
                } else {
                    // The node's own end j: its part within this segment.  The
                    // largest node whose range starts at leaf l > 0 is inner
                    // node l (Karras: the right child of the split between
                    // l - 1 and l is leaf or inner node l), and the largest
                    // ending at r < n - 1 is inner node r, so every crossing
                    // node's suffix suf[l] and prefix pre[r] are written here by
                    // nodes l and r (pre[n - 1] above); the other leaves need
                    // neither.
                    crosses = true;
                    if (gl == j) gstore(suf, j, T.query(t, cnt - 1u));
                    else gstore(pre, j, T.query(0u, t));
                }
            }
        }
    }
    const uint32_t lane = t & 31u, bm = __ballot_sync(0xffffffffu, crosses);
    if (bm != 0u) {
        const int leader = __ffs(bm) - 1;
        uint32_t at = 0;
        if ((int)lane == leader) at = atomicAdd(n_cross, (uint32_t)__popc(bm));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (crosses) cross[at + __popc(bm & ((1u << lane) - 1u))] = j;
    }
}

// Sparse tables over the segment unions: t1 level k entry i at t1 + 6 (k nseg
// + i), built within 256-entry groups (level 0 = the segment unions); t2 the
// full table over the group unions, level k entry i at t2 + 6 (k ngrp + i).
// refit_group builds group g's table and union; the last group to finish
// (ticket) builds t2.  k_refit_top runs it, one block per group.  (Running
// it instead in the last of a group's segment blocks to finish, behind a
// per-group ticket, made every segment block wait for its fence and ticket:
// 1M build 0.215 -> 0.223 ms, 4M 0.871 -> 0.896 ms.)
__device__ __forceinline__ void refit_group(float *__restrict__ t1, uint32_t nseg, float *__restrict__ t2,
                                            uint32_t ngrp, int levels2, uint32_t g, uint32_t *__restrict__ ticket,
                                            float2 (*s_t)[3][kRefitSeg])
{
    SegTable<kRefitLevels> T{s_t};
    const uint32_t t = threadIdx.x, base = g * kRefitSeg, i = base + t;
    const uint32_t cnt = min(kRefitSeg, nseg - base);
    Box6 b{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    if (i < nseg) b = gload_cg(t1, i);
    T.build(b);
    if (i < nseg) {
        for (int k = 1; k < kRefitLevels; ++k) gstore(t1, (size_t)k * nseg + i, T.get(k, t));
    }
    if (t == 0u) gstore(t2, g, T.query(0u, cnt - 1u));
    // the last group to finish builds the table over the group unions
    __threadfence();
    bool last = false;
    if (t == 0u) last = atomicAdd(ticket, 1u) == ngrp - 1u;
    if (!__syncthreads_or(last)) return;
    __threadfence();
    if (ngrp > kMaxGroups) {   // batches beyond 2^25 leaves: level by level through L2
#pragma unroll 1
        for (int k = 1; k < levels2; ++k) {
            const uint32_t half = 1u << (k - 1);
            const float *prev = t2 + 6 * (size_t)(k - 1) * ngrp;
            for (uint32_t e = t; e < ngrp; e += kRefitSeg) {
                Box6 y = gload_cg(prev, e);
                if (e + half < ngrp) y = box_join(y, gload_cg(prev, e + half));
                gstore(t2 + 6 * (size_t)k * ngrp, e, y);
            }
            __threadfence();
            __syncthreads();
        }
        return;
    }
    // the group table in this block's shared memory (two levels of up to
    // kMaxGroups entries in the segment table's space), each level stored out
    float(*lv)[6][kMaxGroups] = reinterpret_cast<float(*)[6][kMaxGroups]>(&s_t[0][0][0].x);
    for (uint32_t e = t; e < ngrp; e += kRefitSeg) {
        const Box6 y = gload_cg(t2, e);
        for (int c = 0; c < 3; ++c) {
            lv[0][c][e] = y.lo[c];
            lv[0][3 + c][e] = y.hi[c];
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int k = 1; k < levels2; ++k) {
        const uint32_t half = 1u << (k - 1);
        const int a = (k - 1) & 1, o = k & 1;
        for (uint32_t e = t; e < ngrp; e += kRefitSeg) {
            Box6 y{{lv[a][0][e], lv[a][1][e], lv[a][2][e]}, {lv[a][3][e], lv[a][4][e], lv[a][5][e]}};
            if (e + half < ngrp) {
                const uint32_t f = e + half;
                y = box_join(y, Box6{{lv[a][0][f], lv[a][1][f], lv[a][2][f]}, {lv[a][3][f], lv[a][4][f], lv[a][5][f]}});
            }
            for (int c = 0; c < 3; ++c) {
                lv[o][c][e] = y.lo[c];
                lv[o][3 + c][e] = y.hi[c];
            }
            gstore(t2 + 6 * (size_t)k * ngrp, e, y);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kRefitSeg)
k_refit_top(float *__restrict__ t1, uint32_t nseg, float *__restrict__ t2, uint32_t ngrp, int levels2,
            uint32_t *__restrict__ ticket)
{
    pdl_enter();
    __shared__ float2 s_t[kRefitLevels][3][kRefitSeg];
    refit_group(t1, nseg, t2, ngrp, levels2, blockIdx.x, ticket, s_t);
}

// the listed inner node at leaf position j, whose range crosses a segment border
template <typename Key, bool BATCH>
__device__ __forceinline__ void refit_cross(const Key *__restrict__ codes, uint32_t n_all, uint32_t j,
                                            const MeshRec *__restrict__ meshes, const uint64_t *__restrict__ keys,
                                            NodeRec *__restrict__ nodes, const uint4 *__restrict__ links,
                                            const uint32_t *__restrict__ parents,
                                            TriRec *__restrict__ tris, RootRec *__restrict__ roots,
                                            const float *__restrict__ pre, const float *__restrict__ suf,
                                            const float *__restrict__ t1, uint32_t nseg, const float *__restrict__ t2,
                                            uint32_t ngrp, uint32_t *__restrict__ flags)
{
    if (j >= n_all) return;
    const MeshSpan sp = mesh_of<BATCH>(j, n_all, meshes, keys);
    const uint32_t jl = j - sp.tri_off;
    uint32_t l, r;
    if (jl + 1u >= sp.n) return;
    const uint4 q3 = links[sp.node_off + jl];
    if (!node_range(q3, sp.n, l, r)) return;
    const uint32_t gl = sp.tri_off + l, gr = sp.tri_off + r, gm = gr + 1u - (q3.w & ~kCollapses);
    const uint32_t sa = gl / kRefitSeg, sb = gr / kRefitSeg;
    if (sa == sb) return;
    Box6 x = gload(suf, gl);
    if (sa + 1u < sb) {
        // segment unions sa + 1 .. sb - 1, in 256-entry groups
        const uint32_t A = sa + 1u, B = sb - 1u, ga = A / kRefitSeg, gb = B / kRefitSeg;
        if (ga == gb) {
            x = box_join(x, t1_query(t1, nseg, A, B));
        } else {
            x = box_join(x, t1_query(t1, nseg, A, ga * kRefitSeg + kRefitSeg - 1u));
            if (ga + 1u < gb) {
                const uint32_t a2 = ga + 1u, b2 = gb - 1u;
                const int k = floor_log2(b2 - a2 + 1u);
                const float *lv = t2 + 6 * (size_t)k * ngrp;
                x = box_join(x, box_join(gload(lv, a2), gload(lv, b2 + 1u - (1u << k))));
            }
            x = box_join(x, t1_query(t1, nseg, gb * kRefitSeg, B));
        }
    }
    x = box_join(x, gload(pre, gr));
    // the node's links (its children write their boxes into its record)
    nodes[sp.node_off + jl].q3 = make_uint4(child_link(q3.z, sp, q3.x, gl, gm - 1u, tris),
                                            child_link(q3.w, sp, q3.y, gm, gr, tris), q3.z & ~kCollapses,
                                            q3.w & ~kCollapses);
    // its box into its parent's record, whose range crosses a border too
    if (jl == 0u) {
        write_root(codes, sp, x, tris, roots);
        return;
    }
    const uint32_t pl = parents[sp.parent_off + jl], p = parent_index(pl);
    if (p >= sp.n - 1u) {
        atomicOr(flags, RTA_DEV_BAD_LINK);
        return;
    }
    write_slot(nodes + sp.node_off + p, pl & 1u, x.lo, x.hi);
}

template <typename Key, bool BATCH>
__global__ void __launch_bounds__(256)
k_refit_ext(const Key *__restrict__ codes, uint32_t n_all, const MeshRec *__restrict__ meshes,
            const uint64_t *__restrict__ keys, NodeRec *__restrict__ nodes, const uint4 *__restrict__ links,
            const uint32_t *__restrict__ parents,
            TriRec *__restrict__ tris, RootRec *__restrict__ roots, const float *__restrict__ pre,
            const float *__restrict__ suf, const float *__restrict__ t1, uint32_t nseg,
            const float *__restrict__ t2, uint32_t ngrp, const uint32_t *__restrict__ cross,
            const uint32_t *__restrict__ n_cross, uint32_t cross_cap, uint32_t *__restrict__ flags)
{
    pdl_enter();
    const uint32_t count = min(*n_cross, cross_cap);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x)
        refit_cross<Key, BATCH>(codes, n_all, cross[e], meshes, keys, nodes, links, parents, tris, roots, pre, suf,
                                t1, nseg, t2, ngrp, flags);
}

} // namespace

// sizes of the refit tables for n leaves (in boxes of 6 floats)
struct RefitLayout {
    uint32_t nseg, ngrp;
    int levels2;
    size_t pre, suf, t1, t2, total;
};
inline RefitLayout refit_layout(uint32_t n)
{
    RefitLayout L;
    L.nseg = (n + kRefitSeg - 1) / kRefitSeg;
    L.ngrp = (L.nseg + kRefitSeg - 1) / kRefitSeg;
    L.levels2 = 1;
    while ((2u << (L.levels2 - 1)) <= L.ngrp) ++L.levels2;
    L.pre = 0;
    L.suf = L.pre + n;
    L.t1 = L.suf + n;
    L.t2 = L.t1 + (size_t)kRefitLevels * L.nseg;
    L.total = L.t2 + (size_t)L.levels2 * L.ngrp;
    return L;
}

// The refit of n_all leaves after the Karras kernel.  With tris_in it also
// gathers the Morton-ordered triangles (ids[j] = input index of sorted
// position j; rewritten local to the mesh in a batch); with tris_in null the
// Karras kernel has written them to tris already.  Tables in rbox
// (refit_layout(n_all).total boxes), the crossing list in cross (one word per
// inner node: cross_cap), *n_cross and *ticket zero on entry.
template <typename Key, bool BATCH>
int refit_launch(const Key *codes, uint32_t n_all, const MeshRec *meshes, const uint64_t *keys,
                 const float *tris_in, uint32_t *ids, NodeRec *nodes, const uint4 *links, const uint32_t *parents,
                 TriRec *tris, RootRec *roots, float *rbox, uint32_t *cross, uint32_t cross_cap, uint32_t *n_cross,
                 uint32_t *ticket, uint32_t *flags, int sms, cudaStream_t s, bool pdl = false)
{
    const RefitLayout L = refit_layout(n_all);
    float *pre = rbox + 6 * L.pre, *suf = rbox + 6 * L.suf, *t1 = rbox + 6 * L.t1, *t2 = rbox + 6 * L.t2;
    cudaError_t e = launch_pdl(pdl, k_refit_seg<Key, BATCH>, dim3(L.nseg), dim3(kRefitSeg), 0, s, codes, n_all,
                               meshes, keys, tris_in, ids, nodes, links, parents, tris, roots, pre, suf, t1, cross,
                               n_cross, flags);
    if (e == cudaSuccess)
        e = launch_pdl(pdl, k_refit_top, dim3(L.ngrp), dim3(kRefitSeg), 0, s, t1, L.nseg, t2, L.ngrp, L.levels2,
                       ticket);
    if (e == cudaSuccess && n_all > 2u) {
        const uint32_t want = (n_all + 255u) / 256u, cap = (uint32_t)sms * 4u;
        e = launch_pdl(pdl, k_refit_ext<Key, BATCH>, dim3(want < cap ? want : cap), dim3(256), 0, s, codes, n_all,
                       meshes, keys, (NodeRec *)nodes, links, parents, tris, roots, (const float *)pre,
                       (const float *)suf, (const float *)t1, L.nseg, (const float *)t2, L.ngrp,
                       (const uint32_t *)cross, (const uint32_t *)n_cross, cross_cap, flags);
    }
    if (e != cudaSuccess) {
        set_cuda_error(e, "refit");
        return RTA_ERR_CUDA;
    }
    return RTA_OK;
}

} // namespace rta
