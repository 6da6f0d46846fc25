// common.cuh -- device layouts and helpers shared by the LBVH build, the
// traversal and the ray kernels (sm_103a).
//
// Device layouts (all 16-byte aligned, sized for vector loads):
//   NodeRec  64 B per inner node i in [0, n-2] (the reference numbers inner
//            nodes 0..n-2 and leaves n-1..2n-2, lbvh-kernels.cu:197-203).  A
//            node stores the boxes and links of BOTH children, so the
//            child-is test of an inner node is one 64-byte fetch.  The
//            planes are interleaved left / right, so each 64-bit half of
//            q0..q2 holds one plane of both children (the operand pair of
//            one paired f32x2 instruction):
//              q0 = (left lo.x, right lo.x, left hi.x, right hi.x)
//              q1 = (left lo.y, right lo.y, left hi.y, right hi.y)
//              q2 = (left lo.z, right lo.z, left hi.z, right hi.z)
//              q3 = (left link, right link, left size, right size)
//            size = number of triangles under the child (its Morton range).
//            A left child's range ends at its node index and a right child's
//            range starts at it (Karras' split), so the reference's node
//            numbering of every child follows from link and size.
//   RootRec  32 B: root box and root link.
//   TriRec   48 B per triangle in Morton order: (a, count), (b, id), (c, 0).
//            count = number of triangles of the leaf that starts here.
//   link     bit 31 clear: inner node index.  Bit 31 set: a leaf,
//            bits 30..25 = min(count, 64) - 1 (63 = look up count in the
//            TriRec), bits 24..0 = first triangle (Morton position).
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "../../include/rta_gb300.h"

namespace rta {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kCountShift = 25;
constexpr uint32_t kCountMask = 0x3fu;
constexpr uint32_t kFirstMask = (1u << kCountShift) - 1u;
constexpr uint32_t kMaxTriangles = 1u << kCountShift;

struct __align__(16) NodeRec {
    float4 q0, q1, q2;
    uint4 q3;
};
static_assert(sizeof(NodeRec) == 64, "node record");

// float offsets in a NodeRec of child `side`'s (0 left, 1 right) planes
__host__ __device__ __forceinline__ int slot_lo(uint32_t side, int axis) { return 4 * axis + (int)side; }
__host__ __device__ __forceinline__ int slot_hi(uint32_t side, int axis) { return 4 * axis + 2 + (int)side; }
// a child's box as the argument list (lo.x, hi.x, lo.y, hi.y, lo.z, hi.z)
#define RTA_LEFT_BOX(nd) (nd).q0.x, (nd).q0.z, (nd).q1.x, (nd).q1.z, (nd).q2.x, (nd).q2.z
#define RTA_RIGHT_BOX(nd) (nd).q0.y, (nd).q0.w, (nd).q1.y, (nd).q1.w, (nd).q2.y, (nd).q2.w

struct __align__(16) RootRec {
    float lo[3], hi[3];
    uint32_t link, pad;
};
static_assert(sizeof(RootRec) == 32, "root record");

struct __align__(16) TriRec {
    float4 v0, v1, v2;
};
static_assert(sizeof(TriRec) == 48, "triangle record");

struct HitRec {
    float t, beta, gamma;
    uint32_t ref;
};

__host__ __device__ __forceinline__ bool is_leaf(uint32_t link) { return (link & kLeafBit) != 0u; }
__host__ __device__ __forceinline__ uint32_t leaf_first(uint32_t link) { return link & kFirstMask; }
__host__ __device__ __forceinline__ uint32_t leaf_count_field(uint32_t link)
{
    return (link >> kCountShift) & kCountMask;
}
__host__ __device__ __forceinline__ uint32_t make_leaf(uint32_t first, uint32_t count)
{
    uint32_t f = count >= 64u ? 63u : count - 1u;
    return kLeafBit | (f << kCountShift) | first;
}

// The reference's MIN / MAX macros (lbvh-kernels.cu:142-143): ternaries, not
// fminf/fmaxf, so that equal-valued signed zeros resolve the same way.
__host__ __device__ __forceinline__ float ref_min(float a, float b) { return (a < b) ? a : b; }
__host__ __device__ __forceinline__ float ref_max(float a, float b) { return (a > b) ? a : b; }

// rays per tile of the bounce compaction kernels (rays.cu); the fused frame
// counts each tile's bounce rays for the gather
constexpr int kBounceTileLog2 = 10;

// Programmatic dependent launch along the build's kernel chain: a kernel
// launched by launch_pdl may start while the previous kernel of its stream
// drains.  Every chained kernel first waits for the previous kernel's
// completion and memory (griddepcontrol.wait) before it touches memory, then
// lets the next kernel launch (griddepcontrol.launch_dependents), which
// happens once all of its own blocks have started.  For a kernel launched
// without the attribute both instructions do nothing.
#ifndef RTA_PDL
#define RTA_PDL 1
#endif
__device__ __forceinline__ void pdl_enter()
{
#if RTA_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Bounded spin: every wait on another block gives up after this many polls
// and raises RTA_DEV_SPIN_TIMEOUT instead of hanging the GPU.
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p)
{
    return *(const volatile uint32_t *)p;
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) { *(volatile uint32_t *)p = v; }

// decoupled look-back status words: 2 flag bits + 30-bit value
constexpr uint32_t kStatAggregate = 1u << 30;
constexpr uint32_t kStatPrefix = 2u << 30;
constexpr uint32_t kStatValue = (1u << 30) - 1u;

// Walks tile statuses backwards from tile-1 until an inclusive prefix is found;
// returns the exclusive prefix of `tile` for one counter.  stat[t * stride]
// is tile t's word.  The words of up to kLookbackWindow predecessors are
// loaded at once (independent loads, one latency) and consumed nearest
// first; a word not yet written ends the window and is polled again.
// Bounded: sets RTA_DEV_SPIN_TIMEOUT in *flags on give-up.
#ifndef RTA_LOOKBACK_WINDOW
#define RTA_LOOKBACK_WINDOW 8
#endif
constexpr int kLookbackWindow = RTA_LOOKBACK_WINDOW;

__device__ __forceinline__ uint32_t lookback(const uint32_t *stat, uint32_t stride, uint32_t tile,
                                             uint32_t *flags)
{
    uint32_t excl = 0;
    int t = (int)tile - 1;
    uint32_t spins = 0;
    while (t >= 0) {
        uint32_t s[kLookbackWindow];
#pragma unroll
        for (int w = 0; w < kLookbackWindow; ++w)
            s[w] = t - w >= 0 ? ld_volatile(stat + (size_t)(t - w) * stride) : 0u;
        int used = 0;
        bool stop = false;
#pragma unroll
        for (int w = 0; w < kLookbackWindow; ++w) {
            if (stop || t - w < 0) break;
            const uint32_t v = s[w];
            if ((v & ~kStatValue) == 0u) {
                stop = true;   // not written yet: poll it again
                break;
            }
            excl += v & kStatValue;
            ++used;
            if (v & kStatPrefix) return excl;
        }
        t -= used;
        if (stop) {
            if (++spins > kSpinLimit) {
                atomicOr(flags, RTA_DEV_SPIN_TIMEOUT);
                break;
            }
            if (used == 0) __nanosleep(32);
        }
    }
    return excl;
}

} // namespace rta

// host-side error helpers (one translation unit defines the storage)
namespace rta {
void set_cuda_error(cudaError_t e, const char *where);
void set_error_message(const char *msg);
int check_launch(const char *where);

// a kernel launch that may overlap the previous kernel of the stream (above)
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = (RTA_PDL && pdl) ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
} // namespace rta

#define RTA_CUDA_TRY(call)                                                                   \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess) {                                                             \
            rta::set_cuda_error(_e, #call);                                                  \
            return _e == cudaErrorMemoryAllocation ? RTA_ERR_NOMEM : RTA_ERR_CUDA;           \
        }                                                                                    \
    } while (0)
