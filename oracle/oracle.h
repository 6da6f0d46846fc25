/*
 * oracle.h -- CPU restatement of the rta LBVH build, binary-BVH traversal,
 * Shirley camera and the added diffuse bounce.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (rta_gb300/, plugin/,
 * include/) links or calls this code: it is imported by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline leg.
 *
 * Every function names the reference file:line whose arithmetic it restates.
 * Compile with -ffp-contract=off: the reference expressions are evaluated as
 * written (no fused multiply-add), which is the arithmetic the GPU path keeps.
 */
#ifndef RTA_ORACLE_H
#define RTA_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One reference triangle record (librta/cuda-vec.h:30-37, 104 bytes): positions
 * a,b,c at float offsets 0..8, then normals, texcoords and an int material. */
#define ORC_TRI_FLOATS 26

/* Reference-layout ("2F4", bbvh-cuda/bbvh-cuda-node.h:37-91) node: 8 floats.
 *   [0] bits: (left<<1)|1 for inner, (elems<<1) for leaf
 *   [1] bits: right child (inner) or first triangle (leaf)
 *   [2..4] box min xyz, [5..7] box max xyz                                  */
#define ORC_NODE_FLOATS 8

/* quirk / event flags reported by orc_lbvh_build */
#define ORC_FLAG_WRAP        1u  /* a quantised axis value reached the grid size and wrapped to 0 */
#define ORC_FLAG_NONFINITE   2u  /* a scene axis has zero extent (scale is inf) */
#define ORC_FLAG_CODE0_RACE  4u  /* code 0 present: the reference refit may drop ancestors */

typedef struct {
    float t, beta, gamma;
    uint32_t ref;
} orc_hit;

/* ---- LBVH (bbvh-cuda/lbvh-kernels.cu, bbvh-cuda/lbvh.h:153-211) ---- */

/* Builds the LBVH of n triangles (records of ORC_TRI_FLOATS floats).
 * morton_bits: 30 (reference, GRIDSIZE 1024) or 63 (21 bits per axis).
 * Outputs (caller allocated):
 *   codes  [n]        sorted Morton codes (uint64 even for 30-bit codes)
 *   ids    [n]        sorted triangle ids (reference index_buffer)
 *   nodes  [(2n-1)*8] reference 2F4 node array
 *   scene  [6]        scene box (min xyz, max xyz) as reduced by the reference
 *   scale  [3]        quantisation scale d = GRIDSIZE/extent
 * Returns 0 on success, negative on bad input. *flags receives ORC_FLAG_*.  */
int orc_lbvh_build(const float *tris, uint32_t n, int morton_bits,
                   uint64_t *codes, uint32_t *ids, float *nodes,
                   float *scene, float *scale, uint32_t *flags);

/* Morton code of one centroid, as morton_codes2 (lbvh-kernels.cu:169-183). */
uint64_t orc_morton(const float c[3], const float mn[3], const float d[3], int morton_bits,
                    uint32_t *flags);

/* Centroid ((a+b)+c)/3.0f (lbvh-kernels.cu:60-63). */
void orc_centroid(const float *tri, float out[3]);

/* Gathers full triangle records into sorted order (lbvh-kernels.cu:557-578). */
void orc_permute(const float *tris, const uint32_t *ids, uint32_t n, float *out);

/* ---- traversal (bbvh-cuda/kernels.cu) ---- */

/* trace modes */
#define ORC_CIS     0   /* child-is, 2F4 (kernels.cu:777-855) */
#define ORC_DIS     1   /* direct-is, 2F4 (kernels.cu:486-548) */
#define ORC_SHADOW  2   /* flag: any-hit early out (kernels.cu:857-939) */
#define ORC_AILA    4   /* flag: Aila box test (intersect.h:165-176, kernels.cu:945-1010) */

/* Traces nrays rays through a reference-layout BVH.
 *   tris  sorted triangle records (ORC_TRI_FLOATS each) indexed by leaf offsets
 *   orig/dir  3 floats per ray, maxt one float per ray (librta/cuda.h:92-100)
 *   hits  in/out: read for the miss case (reference keeps beta/gamma/ref)
 *   stats optional [nrays*2]: inner nodes visited, triangles tested
 * Returns 0, or -1 if some ray overflowed the stack limit.               */
int orc_trace(const float *nodes, const float *tris, const float *orig, const float *dir,
              const float *maxt, uint32_t nrays, int mode, int stack_limit,
              orc_hit *hits, uint32_t *stats, int threads);

/* slab test (librta/intersect.h:56-150); returns hit, *dist = t_near */
int orc_intersect_aabb(const float bmin[3], const float bmax[3], const float o[3],
                       const float d[3], float *dist);
/* triangle test (librta/intersect.h:8-53) */
int orc_intersect_tri(const float *tri, const float o[3], const float d[3],
                      float *t, float *beta, float *gamma);

/* ---- rays (librta/cuda-kernels.cu) ---- */

/* setup_shirley_rays (cuda-kernels.cu:50-112).  tan_half_fovy is the value the
 * reference computes as tanf(M_PI*(fovy/2)/180.0f); passing it in keeps the
 * rays bit-identical across machines whose tanf differ.                   */
void orc_shirley_rays(float *dirs, float *orgs, float *maxts, float tan_half_fovy,
                      float aspect, int w, int h, const float view_dir[3],
                      const float pos[3], const float up[3], float maxt);

/* reset_intersections (cuda-kernels.cu:24-44): t=FLT_MAX, beta=1, gamma=2 */
void orc_reset_hits(orc_hit *hits, uint32_t n);

/* Added (not in the reference): one cosine-weighted diffuse bounce ray per
 * hit, compacted in ray order.  Returns the number of bounce rays.         */
uint32_t orc_diffuse_bounce(const float *tris, const float *orig, const float *dir,
                            const orc_hit *hits, uint32_t nrays, uint32_t seed, float eps,
                            float *out_orig, float *out_dir, float *out_maxt,
                            uint32_t *out_src);

/* uniform random float in [0,1) for (seed, index) -- shared with the GPU */
float orc_uniform(uint32_t seed, uint32_t index);
/* cos and sin of 2*pi*u, u in [0,1) -- shared with the GPU */
void orc_cos_sin_2pi(float u, float *c, float *s);

/* ---- CPU bbvh plugin (bbvh/bbvh.h:110-279, 382-460) ---- */

/* Spatial-median binary BVH (bbvh_constructor_using_median, max 4 tris/leaf).
 * tris is sorted in place by the build (qsort as the reference does);
 * out_tris receives the leaf-ordered triangle copy; nodes are 32-byte
 * bbvh_node records (2 uint32 + box) = 8 floats.  Returns node count or <0. */
int64_t orc_bbvh_build(float *tris, uint32_t n, float *out_tris, float *nodes, uint32_t max_nodes);

/* bbvh_child_is_tracer::trace_ray, OpenMP over rays. */
int orc_bbvh_trace_cis(const float *nodes, const float *tris, const float *orig,
                       const float *dir, const float *maxt, uint32_t nrays,
                       orc_hit *hits, int threads);

/* ---- host shading (librta/raytrav.h:174-243) ---- */

/* lighting_collector::reset(bg) (bg may be NULL: no reset) then ::shade(binary)
 * over the w x h hits: Lambert point lights with barycentric-interpolated
 * vertex normals; tris are the 26-float records the hits' ref indexes;
 * lights are nl * (position xyz, colour rgb); img is w*h*3 bytes. */
void orc_shade_lambert(const float *tris, const orc_hit *hits, uint32_t w, uint32_t h,
                       const float *lights, uint32_t nl, int binary, const float *bg,
                       uint8_t *img);

#ifdef __cplusplus
}
#endif
#endif
