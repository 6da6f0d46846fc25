// batch.cuh -- device layout of a batch of meshes, shared by the batched
// build (batch.cu) and the batched trace kernel (trace.cu).
//
// The meshes' data lie in one allocation per kind, each mesh in its own
// contiguous range, so a mesh's tree is exactly the one-mesh layout
// (common.cuh) at an offset: links, triangle ids and hit refs are local to
// the mesh.
//   triangles / codes / ids    [tri_off, tri_off + n)
//   inner nodes / counters     [node_off, node_off + n - 1),  node_off = tri_off - m
//   parent words               [parent_off, parent_off + 2n - 1),  parent_off = 2 tri_off - m
//   root                       roots[m]
//   rays / hits                [ray_off, ray_off + rays)
#pragma once

#include "common.cuh"

namespace rta {

struct __align__(16) MeshRec {
    uint32_t tri_off, n_tris, node_off, parent_off;
    uint32_t ray_off, n_rays, pad0, pad1;
};
static_assert(sizeof(MeshRec) == 32, "mesh record");

// the mesh whose prefix range holds element i: the last m with off[m] <= i
// (off has count + 1 entries, off[0] = 0; empty ranges are skipped)
__device__ __forceinline__ uint32_t find_range(const uint32_t *__restrict__ off, uint32_t count, uint32_t i)
{
    uint32_t lo = 0, hi = count;   // answer in [lo, hi)
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

struct BatchTraceArgs {
    const NodeRec *nodes;
    const RootRec *roots;
    const TriRec *tris;
    const MeshRec *meshes;
    const uint32_t *ray_off;   // meshes + 1 entries
    uint32_t n_meshes;
    const float *orig, *dir, *maxt;
    uint32_t nrays;            // all meshes
    HitRec *hits;
    uint32_t *stats;
    uint32_t *queue;           // zero at launch
    uint32_t *status;
    int fetch_idle;
};

// launches the batched child-is trace (trace.cu)
int launch_batch_trace(const BatchTraceArgs &a, int stack, int blocks_per_sm, cudaStream_t s);
// the occupancy limit of the trace kernel with that stack (blocks per SM);
// also fills the launch-shape caches of every variant, so that a later launch
// inside a graph capture makes no occupancy query
int batch_trace_max_blocks_per_sm(int stack);

} // namespace rta
