// lbvh.cuh -- device pieces of the LBVH build shared by the one-mesh builder
// (build.cu) and the batched multi-mesh builder (batch.cu): build constants,
// position loads, Morton helpers, the onesweep radix pass, Karras' split
// search, the per-node link writer and the bottom-up refit climb.
#pragma once

#include <utility>

#include "common.cuh"

namespace rta {

// ------------------------------------------------------------------------- //
// build state                                                                //
// ------------------------------------------------------------------------- //

constexpr int kTriFloats = 26;         // cuda::simple_triangle = 104 bytes
constexpr int kBoundsThreads = 256;
constexpr int kSortThreads = 256;      // 8 warps
constexpr int kSortItems = 16;
// blocks per SM the onesweep kernel must fit in registers: 3 caps the 64-bit
// key passes at 80 registers (from 128: 2 blocks per SM) at a few spilled
// bytes, 1.5 % off the 4M build; 12 or 8 keys per thread measured slower
#ifndef RTA_SORT_MIN_BLOCKS
#define RTA_SORT_MIN_BLOCKS 3
#endif
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per tile
constexpr int kMaxDigitBits = 11;
constexpr int kMaxRadix = 1 << kMaxDigitBits;
constexpr int kMaxPasses = 8;          // 63-bit keys at 8 bits per digit

struct BuildState {
    float lo[3], hi[3], scale[3];
    uint32_t done;                 // bounds last-block ticket (self-resetting)
    uint32_t refit_done;           // refit summary last-block ticket (self-resetting)
};

// Zeroed by one memset before every build.  hist holds the global digit
// histogram of pass p at hist[p * radix], radix = 2^digit bits.
struct SortScratchHeader {
    uint32_t tile_ctr[kMaxPasses];
    uint32_t hist[kMaxPasses * kMaxRadix];
    uint32_t n_cross;   // refit: inner nodes whose range crosses a segment border
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

// ------------------------------------------------------------------------- //
// one onesweep LSD radix pass                                                 //
// ------------------------------------------------------------------------- //
//
// A tile of 4096 keys per block: warp-level stable ranking with one ballot
// per digit bit, per-warp digit counters in shared memory, decoupled
// look-back across tiles for the per-digit prefix (Merrill & Garland's
// single-pass scan as used by Adinets & Merrill's Onesweep), a shared-memory
// staging of the tile in digit order, and coalesced runs out to global
// memory.  BITS is the digit width (8, 10 or 11): wider digits mean fewer
// passes but larger per-warp counters and more look-back work per tile.

template <typename Key, int BITS>
struct SortSmem {
    static constexpr int kRadix = 1 << BITS;
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
    constexpr int kRadix = 1 << BITS;
    constexpr uint32_t kDigitMask = (uint32_t)kRadix - 1u;
    constexpr int kDpt = kRadix > kSortThreads ? kRadix / kSortThreads : 1;   // digits per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem<Key, BITS> &S = *reinterpret_cast<SortSmem<Key, BITS> *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;

    if (tid == 0) S.tile = atomicAdd(tile_ctr, 1u);
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
        dig[i] = (uint32_t)(k[i] >> shift) & kDigitMask;
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t d = dig[i];
        uint32_t peers = 0xffffffffu;
#pragma unroll
        for (int b = 0; b < BITS; ++b) {
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

    // per digit (thread tid owns digits tid*kDpt .. tid*kDpt+kDpt-1): warp
    // offsets, tile count, block offsets
    uint32_t cnt[kDpt], gh[kDpt];
    uint32_t csum = 0, gsum = 0;
    // padding keys (beyond n) are all the last digit and sit at the end of the last tile
    const uint32_t valid = n - base < (uint32_t)kSortTile ? n - base : (uint32_t)kSortTile;
    const uint32_t pad = (uint32_t)kSortTile - valid;
#pragma unroll
    for (int j = 0; j < kDpt; ++j) {
        const int d = tid * kDpt + j;
        cnt[j] = 0;
        gh[j] = 0;
        if (d < kRadix) {
#pragma unroll
            for (int q = 0; q < kSortThreads / 32; ++q) {
                uint32_t c = S.whist[q][d];
                S.whist[q][d] = cnt[j];
                cnt[j] += c;
            }
            gh[j] = hist[d];
            const uint32_t cv = (d == kRadix - 1) ? cnt[j] - pad : cnt[j];
            uint32_t *my_stat = tstat + (size_t)tile * kRadix + d;
            st_volatile(my_stat, (tile == 0 ? kStatPrefix : kStatAggregate) | cv);
        }
        csum += cnt[j];
        gsum += gh[j];
    }
    uint32_t start = block_excl_scan(csum, S.scan_tmp);
    uint32_t gexcl = block_excl_scan(gsum, S.scan_tmp);
#pragma unroll
    for (int j = 0; j < kDpt; ++j) {
        const int d = tid * kDpt + j;
        if (d < kRadix) {
            const uint32_t cv = (d == kRadix - 1) ? cnt[j] - pad : cnt[j];
            uint32_t excl = 0;
            if (tile > 0) {
                excl = lookback(tstat + d, kRadix, tile, flags);
                __threadfence();
                st_volatile(tstat + (size_t)tile * kRadix + d, kStatPrefix | ((excl + cv) & kStatValue));
            }
            S.digit_start[d] = start;
            S.glob[d] = gexcl + excl - start;
        }
        start += cnt[j];
        gexcl += gh[j];
    }
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
        uint32_t dst = S.glob[(uint32_t)(key >> shift) & kDigitMask] + j;
        kout[dst] = key;
        vout[dst] = S.vals[j];
        if (code_out) code_out[dst] = (uint32_t)key & code_mask;
    }
}

// Launches the P passes of one LSD sort of n keys with BITS-bit digits.  The
// header's tile counters and histograms (filled by the Morton kernel) and the
// tile status words are zero on entry.  On return *keys_sorted / *vals_sorted
// point at the buffers holding the result (ping-pong between the two pairs).
template <typename Key, int BITS>
int sort_passes_launch(Key *k0, Key *k1, uint32_t *v0, uint32_t *v1, uint32_t n, int passes,
                       SortScratchHeader *hdr, uint32_t *tstat, uint32_t *flags, uint32_t *code_out,
                       uint32_t code_mask, cudaStream_t s, Key **keys_sorted, uint32_t **vals_sorted)
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
        k_onesweep<Key, BITS><<<tiles, kSortThreads, smem, s>>>(
            kin, vin, kout, vout, n, BITS * p, hdr->tile_ctr + p, hdr->hist + (size_t)p * kRadix, ts, flags,
            p == passes - 1 ? code_out : nullptr, code_mask);
        int rc = check_launch("k_onesweep");
        if (rc) return rc;
        std::swap(kin, kout);
        vin = vout;
        vout = (vout == v0) ? v1 : v0;
    }
    *keys_sorted = kin;
    *vals_sorted = vin;
    return RTA_OK;
}

} // namespace

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

// links of inner node i (i + 1 < n) of a tree over codes[0, n), its
// children's parent words, and its refit counter
template <typename Key>
__device__ __forceinline__ void karras_node(const Key *__restrict__ codes, uint32_t n, uint32_t i,
                                            NodeRec *__restrict__ nodes, uint32_t *__restrict__ parents,
                                            uint32_t *__restrict__ counters)
{
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
// bottom-up refit                                                             //
// ------------------------------------------------------------------------- //
//
// One thread per leaf climbs towards the root; the second thread to arrive at
// a node (counted with an acquire-release atomic add)
// unions the two child boxes, applies the reference's collapse rule (both
// children leaves with equal Morton codes -> one multi-triangle leaf,
// :300-331) and continues.  A node's box is stored in its parent's record.

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

__device__ __forceinline__ void read_slot_cg(const NodeRec *nd, uint32_t side, float lo[3], float hi[3])
{
    const float *f = reinterpret_cast<const float *>(nd);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = __ldcg(f + slot_lo(side, k));
        hi[k] = __ldcg(f + slot_hi(side, k));
    }
}

// Arrival count with acquire-release semantics at device scope: the first
// arriver's box and link writes (program-ordered before it) are released by
// it, and the second arriver acquires them before it reads the sibling slot.
// One instruction instead of a fence on both sides of a relaxed atomicAdd.
__device__ __forceinline__ uint32_t arrive_acq_rel(uint32_t *p)
{
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

__device__ __forceinline__ uint32_t leaf_count_cg(uint32_t link, const TriRec *tris)
{
    uint32_t f = leaf_count_field(link);
    if (f < 63u) return f + 1u;
    return __float_as_uint(__ldcg(&tris[leaf_first(link)].v0.w));
}

// the climb of leaf j of a tree over codes[0, n)
template <typename Key>
__device__ __forceinline__ void refit_climb(const Key *__restrict__ codes, uint32_t n, uint32_t j,
                                            NodeRec *__restrict__ nodes, const uint32_t *__restrict__ parents,
                                            uint32_t *__restrict__ counters, TriRec *__restrict__ tris,
                                            RootRec *__restrict__ root, uint32_t *__restrict__ flags)
{
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
        if (arrive_acq_rel(counters + p) == 0u) return;   // first arrival stops
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

} // namespace rta
