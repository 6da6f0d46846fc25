/*
 * rta_gb300.h -- C ABI of the GB300 LBVH builder and binary-BVH tracer.
 *
 * Plain C: device pointers, sizes and a CUDA stream; every call returns an
 * int status (RTA_OK or a negative RTA_ERR_*), never exits the process.  The
 * rta plugin (plugin/bbvh_gb300.cpp) converts a failure into the reference's
 * behaviour (print and exit, librta/cuda.h:70-77) at the plugin boundary.
 *
 * Each entry point names the reference function it replaces (kiselgra/rta,
 * path:line).  Host-visible layouts that cross this boundary are the
 * reference's:
 *   triangles  cuda::simple_triangle, 104 bytes (librta/cuda-vec.h:30-37),
 *              positions a,b,c at byte offsets 0..35
 *   rays       origin float[3*n], direction float[3*n], max_t float[n]
 *              (librta/cuda.h:90-107)
 *   hits       triangle_intersection {float t, beta, gamma; uint ref},
 *              16 bytes (librta/basic_types.h:81-95); ref indexes the
 *              Morton-ordered triangle array, miss <=> t == FLT_MAX
 *   2F4 nodes  bbvh_node_float4 (bbvh-cuda/bbvh-cuda-node.h:37-91), only
 *              produced on request for dumps and parity checks
 */
#ifndef RTA_GB300_H
#define RTA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *rta_stream_t; /* a cudaStream_t; NULL = legacy default stream */

/* ---- status codes ---- */
#define RTA_OK 0
#define RTA_ERR_INVALID (-1)     /* bad argument (null pointer, n == 0, size limit) */
#define RTA_ERR_CUDA (-2)        /* a CUDA runtime call failed; see rta_last_error() */
#define RTA_ERR_DEVICE (-3)      /* a kernel raised a device status flag */
#define RTA_ERR_NOMEM (-4)       /* device allocation failed */

/* device status flags (rta_lbvh_status, rta_frame_status) */
#define RTA_DEV_STACK_OVERFLOW 1u  /* a ray's traversal stack overflowed; that ray is unfinished */
#define RTA_DEV_SPIN_TIMEOUT 2u    /* a bounded wait in a single-pass scan gave up */
#define RTA_DEV_QUANT_WRAP 4u      /* a quantised centroid reached the grid size and wrapped (reference quirk, kept) */
#define RTA_DEV_ZERO_EXTENT 8u     /* a scene axis has zero extent (scale is inf, reference quirk, kept) */
#define RTA_DEV_ITER_LIMIT 16u     /* a traversal or refit loop hit its iteration cap and stopped */
#define RTA_DEV_BAD_LINK 32u       /* a node link or triangle index was out of range; the access was skipped */

/* trace modes: rta plugin flags -t dis|cis, -s, -A (bbvh-cuda/main.cpp:40-51) */
#define RTA_TRACE_CIS 0u     /* child-is closest hit (kernels.cu:777-855) */
#define RTA_TRACE_DIS 1u     /* direct-is (kernels.cu:486-548) */
#define RTA_TRACE_SHADOW 2u  /* any hit: stop at the first accepted hit (kernels.cu:857-939) */
#define RTA_TRACE_AILA 4u    /* Aila-Laine reciprocal box test (intersect.h:165-176) */
#define RTA_TRACE_STATS 8u   /* also write per-ray counts {inner nodes visited, triangles tested} */

/* Message of the last failing CUDA call in this thread ("" if none). */
const char *rta_last_error(void);

/* Largest triangle count one LBVH may hold (leaf links carry 25-bit offsets). */
uint32_t rta_lbvh_max_triangles(void);

/* ------------------------------------------------------------------------ */
/* LBVH construction -- replaces lbvh_constructor (bbvh-cuda/lbvh.h:49-216)  */
/* ------------------------------------------------------------------------ */

typedef struct rta_lbvh_ctx rta_lbvh_ctx;

/* Device view of a built LBVH.  All pointers are device pointers owned by
 * the context; they stay valid until the next build or reserve. */
typedef struct rta_lbvh {
    const void *nodes;       /* (n-1) inner-node records, 64 bytes each */
    const void *root;        /* root record, 32 bytes: box min xyz, max xyz, link, pad */
    const void *tris;        /* n Morton-ordered triangles, 48 bytes each */
    const uint32_t *index;   /* n: Morton position -> input triangle id (lbvh.h:20-28) */
    const void *codes;       /* n sorted Morton codes: uint32 (30-bit) or uint64 (63-bit) */
    const uint32_t *parents; /* 2n-1 parent links ((parent << 1) | side), reference numbering;
                                bit 31 set when the parent's Morton range crosses a
                                256-leaf border (build bookkeeping: mask it off) */
    uint32_t n;
    int32_t morton_bits;
    uint32_t *status;        /* device word of RTA_DEV_* flags */
    void *ready;             /* a cudaEvent_t recorded on the build's stream after the
                              * last build of this tree (NULL for batch meshes):
                              * calls that read the tree on streams of their own
                              * (rta_host_frames_run) wait for it */
} rta_lbvh;

/* new/delete of lbvh_constructor (lbvh.h:114-145) */
int rta_lbvh_create(rta_lbvh_ctx **ctx);
int rta_lbvh_destroy(rta_lbvh_ctx *ctx);

/* setupCudaMemory (lbvh-kernels.cu:368-383): sizes the device buffers for up to
 * n triangles; build() calls it when n grows, as buildCUDA does (lbvh.h:157-162). */
int rta_lbvh_reserve(rta_lbvh_ctx *ctx, uint32_t n, int morton_bits);

/* Radix digit width of the build's key sort: 8 (default), 9, 10 or 11 bits
 * per pass.  The sorted order is the same for every width (a stable LSD sort);
 * wider digits take fewer passes.  The reference sorts with thrust
 * (sortMortonCodes, lbvh-kernels.cu:537-555), which picks its own width. */
int rta_lbvh_set_digit_bits(rta_lbvh_ctx *ctx, int digit_bits);

/* lbvh_constructor::buildCUDA (lbvh.h:153-211): initTriangles,
 * calculateVoxelBounds, calculateMortonCodes2, sortMortonCodes,
 * buildTreeKarras, buildBoundingBoxesKarras2, invert_triangle_permutation_cuda
 * (lbvh-kernels.cu:405-578), as one stream-ordered sequence with no host sync.
 *   tris       n input triangles (device, 104 bytes each); not modified
 *   morton_bits 30 (the reference's 10 bits per axis) or 63 (21 bits per axis)
 *   tris_out   optional (nullable): receives the input records gathered into
 *              Morton order, the array the reference writes back into its
 *              input buffer and indexes with triangle_intersection::ref */
int rta_lbvh_build(rta_lbvh_ctx *ctx, const void *tris, uint32_t n, int morton_bits,
                   void *tris_out, rta_stream_t stream);

/* Per-pass build timing, as lbvh_constructor::buildCUDA prints it under -v
 * (lbvh.h:172-204): with timing on, rta_lbvh_build records CUDA events on its
 * stream between its passes, and rta_lbvh_pass_ms waits for the last build's
 * end and writes the milliseconds of each pass, in this order:
 *   0  triangle boxes, centroids and the scene box (initTriangles +
 *      calculateVoxelBounds)
 *   1  Morton codes and the sort's digit histograms (calculateMortonCodes2)
 *   2  the key sort (sortMortonCodes)
 *   3  Karras radix tree and parent links (buildTreeKarras)
 *   4  node boxes, equal-code collapse and the Morton-ordered triangles
 *      (buildBoundingBoxesKarras2 + invert_triangle_permutation)
 * Invalid before a timed build.  The events end the overlap of consecutive
 * launches at the pass borders, so a timed build is slightly slower. */
#define RTA_LBVH_PASSES 5
int rta_lbvh_set_timing(rta_lbvh_ctx *ctx, int on);
int rta_lbvh_pass_ms(rta_lbvh_ctx *ctx, float *ms);

/* the built tree: binary_lbvh::take_node_array / take_index_array (lbvh.h:207-208) */
int rta_lbvh_get(const rta_lbvh_ctx *ctx, rta_lbvh *out);

/* Synchronises the stream and returns the device status flags (RTA_DEV_*). */
int rta_lbvh_status(const rta_lbvh *bvh, rta_stream_t stream, uint32_t *flags);

/* Self-test of the bounded waits: one small kernel runs the single-pass
 * scans' look-back against a predecessor status word that nothing writes,
 * so every wait gives up at its poll limit (about a second) instead of
 * hanging.  Returns the device flags it raised in *flags (RTA_DEV_SPIN_TIMEOUT
 * expected); the context stays usable.  Synchronises the stream. */
int rta_selftest_bounded_wait(rta_stream_t stream, uint32_t *flags);

/* Writes the tree in the reference's 2F4 node layout ((2n-1) x 32 bytes),
 * node for node as buildTreeKarras + buildBoundingBoxesKarras2 leave it, for
 * dumps (bbvh.h:36-52) and parity checks. */
int rta_lbvh_to_2f4(const rta_lbvh *bvh, void *nodes_2f4, rta_stream_t stream);

/* ------------------------------------------------------------------------ */
/* traversal -- replaces trace_cis / trace_dis / trace_shadow_* / *_ailabox  */
/* (bbvh-cuda/kernels.cu:1145-1338, host launchers)                          */
/* ------------------------------------------------------------------------ */

/* Traces nrays rays (or *d_nrays if d_nrays is not NULL, read on the device)
 * through bvh.  hits: nrays records; a hit overwrites the record, a miss
 * writes only t = FLT_MAX (the reference keeps beta/gamma/ref of the
 * record, kernels.cu:794-796).  stats: optional, 2 uint32 per ray when
 * RTA_TRACE_STATS is set.  Rays are fetched in warp batches from a global
 * queue by a persistent grid. */
int rta_trace(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt,
              uint32_t nrays, const uint32_t *d_nrays, void *hits, uint32_t mode,
              uint32_t *stats, rta_stream_t stream);

/* ------------------------------------------------------------------------ */
/* rays -- librta/cuda-kernels.cu                                            */
/* ------------------------------------------------------------------------ */

/* setup_shirley_rays (cuda-kernels.cu:50-112).  tan_half_fovy is the value the
 * reference kernel computes as tanf(M_PI*(fovy/2)/180.0f); the caller passes
 * it (cuda::cam_ray_generator_shirley computes it once per frame). */
int rta_setup_shirley_rays(float *dirs, float *orgs, float *maxts, float tan_half_fovy,
                           float aspect, int w, int h, const float view_dir[3],
                           const float pos[3], const float up[3], float maxt,
                           rta_stream_t stream);

/* reset_intersections (cuda-kernels.cu:24-44): t = FLT_MAX, beta = 1, gamma = 2. */
int rta_reset_intersections(void *hits, uint32_t w, uint32_t h, rta_stream_t stream);

/* ------------------------------------------------------------------------ */
/* frame: primary trace + one diffuse bounce (no reference counterpart: the  */
/* reference's cuda bouncers never trace further, cuda.h:208-220)            */
/* ------------------------------------------------------------------------ */

typedef struct rta_frame_ctx rta_frame_ctx;

/* Device view of a frame's bounce pass. */
typedef struct rta_frame {
    float *orig, *dir, *maxt;  /* bounce rays, compacted in primary ray order */
    uint32_t *src;             /* primary ray index of each bounce ray */
    void *hits;                /* bounce hits, 16 bytes each */
    uint32_t *count;           /* device: number of bounce rays */
    uint32_t capacity;
} rta_frame;

int rta_frame_create(rta_frame_ctx **ctx, uint32_t max_rays);
int rta_frame_destroy(rta_frame_ctx *ctx);
int rta_frame_get(const rta_frame_ctx *ctx, rta_frame *out);

/* One cosine-weighted diffuse bounce ray per primary hit, compacted in ray
 * order by a single-pass scan: origin = hit point pushed eps along the
 * geometric normal (facing the incoming ray), direction from the seeded
 * uniform pair (seed, 2i) and (seed, 2i+1), max_t = FLT_MAX. */
int rta_diffuse_bounce(rta_frame_ctx *ctx, const rta_lbvh *bvh, const float *orig,
                       const float *dir, const void *hits, uint32_t nrays, uint32_t seed,
                       float eps, rta_stream_t stream);

/* Whole frame: reset primary hits, trace primary rays, generate the bounce,
 * reset bounce hits, trace the bounce rays.  No host synchronisation.
 * orig/dir/maxt/hits are device-addressable: device memory, or pinned host
 * memory under unified addressing (then read and written over the host
 * link; for frames on host buffers rta_host_frames_run is faster). */
int rta_frame_run(rta_frame_ctx *ctx, const rta_lbvh *bvh, const float *orig, const float *dir,
                  const float *maxt, uint32_t nrays, void *hits, uint32_t mode, uint32_t seed,
                  float eps, rta_stream_t stream);

/* Synchronises and returns the frame's device status flags. */
int rta_frame_status(rta_frame_ctx *ctx, rta_stream_t stream, uint32_t *flags);

/* Per-pass timing, as basic_raytracer::timings records it (librta/raytrav.h:
 * 426): with timing on, rta_frame_run records CUDA events on its stream around
 * the frame's trace work (the fused trace launch of a child-is frame; primary
 * trace to bounce trace otherwise; the bounce gather is not included), and
 * rta_frame_trace_ms waits for the last run's end event and returns the
 * milliseconds between them.  Invalid before a timed run. */
int rta_frame_set_timing(rta_frame_ctx *ctx, int on);
int rta_frame_trace_ms(rta_frame_ctx *ctx, float *ms);

/* Frames on host buffers (no counterpart in the reference, whose frames
 * start and end in device memory; its driver downloads the hits, see
 * primary_intersection_downloader, librta/cuda.h:222-245).  Each run copies
 * the rays in, runs rta_frame_run and copies the primary hits, the bounce
 * hits and the bounce count out, on three internal streams with two sets of
 * device buffers used in turn, so consecutive calls overlap one frame's
 * copies with the neighbouring frames' traversal.  Host pointers must be
 * pinned (cudaHostAlloc / cudaHostRegister).  The rays must be in host memory
 * when the call is made; the frame's traversal waits for bvh->ready, so a
 * tree built on `stream` (or any stream) just before the call is complete
 * before it is read; the outputs are complete once `stream` passes the
 * point where the call left it (the call makes `stream` wait for them), so
 * work queued on `stream` afterwards, a rebuild of the tree included, runs
 * after this frame.
 * h_bounce_hits needs room for nrays records: all nrays are written, the
 * first *h_bounce_count of them are the frame's bounce hits.  Two frames may be in flight; a third waits on the GPU for
 * its buffers, not on the host. */
typedef struct rta_host_frames rta_host_frames;
int rta_host_frames_create(rta_host_frames **out, uint32_t max_rays);
int rta_host_frames_destroy(rta_host_frames *frames);
int rta_host_frames_run(rta_host_frames *frames, const rta_lbvh *bvh, const float *h_orig,
                        const float *h_dir, const float *h_maxt, uint32_t nrays, void *h_hits,
                        void *h_bounce_hits, uint32_t *h_bounce_count, uint32_t mode, uint32_t seed,
                        float eps, rta_stream_t stream);

/* No counterpart in the reference.  rta_diffuse_bounce for callers that may
 * not allocate device memory: a renderer that hands all device memory to its
 * own pool under a fixed budget, or a frame loop that must not take
 * cudaMalloc's implicit device synchronisation between two passes.  It calls
 * no cudaMalloc, cudaFree or other allocating routine; its scratch (the
 * look-back words of the ordered compaction) is a 64 KiB module array that
 * every GPU loading the library holds until the process exits.
 *   out_orig/out_dir/out_maxt/out_src  room for nrays bounce rays
 *   out_count  device word: the number of bounce rays written
 *   out_flags  optional device word (nullable): the call's RTA_DEV_* flags;
 *              RTA_DEV_SPIN_TIMEOUT means a bounded wait of the ordered
 *              compaction gave up and the count and ray order are not valid
 * nrays above RTA_BOUNCE_NOALLOC_MAX_RAYS returns RTA_ERR_INVALID with a
 * message in rta_last_error().  The first call on a device (and the first
 * after its context was destroyed and created again) looks up the scratch's
 * device address; make that first call before any stream capture.
 * Every call shares the scratch: calls that overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller. */
#define RTA_BOUNCE_NOALLOC_MAX_RAYS (1u << 24)
int rta_diffuse_bounce_noalloc(const rta_lbvh *bvh, const float *orig, const float *dir,
                               const void *hits, uint32_t nrays, uint32_t seed, float eps,
                               float *out_orig, float *out_dir, float *out_maxt, uint32_t *out_src,
                               uint32_t *out_count, uint32_t *out_flags, rta_stream_t stream);

/* ------------------------------------------------------------------------ */
/* learned child order (no reference counterpart): a 14-32-32-1 network      */
/* that picks which child to visit first where the child-is traversal hits   */
/* both children; trained on decisions recorded from the plain traversal     */
/* ------------------------------------------------------------------------ */

typedef struct rta_order_model rta_order_model;

/* Network (Glorot-uniform from `seed`), optimiser state and room for
 * max_samples training samples (64 bytes each on the device). */
int rta_order_create(rta_order_model **model, uint32_t max_samples, uint32_t seed);
int rta_order_destroy(rta_order_model *model);
/* number of network parameters: w1 (32x16), b1, w2 (32x32), b2, w3, b3 as fp32 */
uint32_t rta_order_param_count(void);
int rta_order_get_params(const rta_order_model *model, float *host_params);
int rta_order_set_params(rta_order_model *model, const float *host_params);
/* Confidence margin of rta_trace_learned (default 0): the network's choice is
 * taken only where |logit| > margin, the plain nearer-first order elsewhere.
 * A margin of FLT_MAX or more gives the plain traversal, and rta_trace_learned
 * then runs the plain child-is kernel without evaluating the network. */
int rta_order_set_margin(rta_order_model *model, float margin);
int rta_order_get_margin(const rta_order_model *model, float *margin);

/* Plain child-is closest-hit trace (as rta_trace with RTA_TRACE_CIS) that
 * also records every node where both children are hit and not culled, then
 * labels those samples from the final hits; successive calls append until
 * max_samples are held. */
int rta_order_sample(rta_order_model *model, const rta_lbvh *bvh, const float *orig,
                     const float *dir, const float *maxt, uint32_t nrays, const uint32_t *d_nrays,
                     void *hits, rta_stream_t stream);
int rta_order_sample_count(const rta_order_model *model, uint32_t *count);
int rta_order_clear_samples(rta_order_model *model);
/* device pointer to the sample records (for inspection) */
int rta_order_samples(const rta_order_model *model, void **d_samples);

/* Gradient of the mean weighted binary cross-entropy over samples
 * [first, first+count) at the current parameters; no update. */
int rta_order_gradient(rta_order_model *model, uint32_t first, uint32_t count, float *host_grad,
                       float *host_loss);
/* Adam over the held samples, `epochs` passes of minibatches of `batch`. */
int rta_order_train(rta_order_model *model, uint32_t epochs, uint32_t batch, float lr,
                    float *last_loss, rta_stream_t stream);

/* Child-is closest-hit trace whose two-child order comes from the network
 * where both children are hit and their entry-exit intervals overlap (the
 * plain nearer-first order elsewhere).  Every child whose rounded entry
 * distance is below the current t is still visited, so each ray hits iff it
 * hits in the plain order, and t agrees up to a few ulps: a triangle's
 * rounded t can lie just below its box's rounded entry, and of two hits that
 * close the order decides which survives.  Of two triangles at exactly the
 * same t another one may be reported.  stats as in rta_trace (nullable). */
int rta_trace_learned(const rta_lbvh *bvh, const rta_order_model *model, const float *orig,
                      const float *dir, const float *maxt, uint32_t nrays, const uint32_t *d_nrays,
                      void *hits, uint32_t *stats, rta_stream_t stream);

/* The ideal child order, as a bound on what any learned order can gain: the
 * trace of rta_trace_learned with each decision taken by known_hits (the
 * ray's closest hit from an earlier trace, 16-byte records as rta_trace
 * writes them): the child whose Morton range holds the hit triangle first.
 * No counterpart in the reference. */
int rta_trace_ideal_order(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt,
                          uint32_t nrays, const void *known_hits, void *hits, uint32_t *stats,
                          rta_stream_t stream);

/* Host shading on the device: lighting_collector::reset and ::shade
 * (librta/raytrav.h:186-233), which the reference runs on the host over
 * downloaded hits (cuda::direct_diffuse_illumination, librta/cuda.h:247-266).
 * Writes the w*h*3-byte RGB image (row-major, as rta's image<unsigned char, 3>)
 * byte for byte as the host shader would:
 *   hits        w*h hit records of a primary pass (device)
 *   tris        the 104-byte records the hits' ref indexes, i.e. the Morton-
 *               ordered array rta_lbvh_build writes to tris_out (device;
 *               unused when binary_only)
 *   lights      n_lights <= 16 point lights, 6 floats each: position, colour
 *               (host); shade() does nothing without lights
 *   binary_only every hit pixel gets the first light's colour
 *   background  host float[3] or NULL: reset(c) first, min(int(c*255), 255)
 *   d_flags     optional device word: RTA_DEV_BAD_LINK if a ref is >= n_tris */
int rta_shade_lambert(const void *hits, const void *tris, uint32_t n_tris, uint32_t w, uint32_t h,
                      const float *lights, uint32_t n_lights, int binary_only, const float *background,
                      void *image, uint32_t *d_flags, rta_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Batched multi-mesh build and trace                                        */
/* ------------------------------------------------------------------------ */
/* Many independent meshes, each with its own 30-bit LBVH over its own box and
 * its own rays, built and traced together: one sort of (mesh id, Morton code)
 * keys, the Karras trees and refits of all meshes in one launch each, and one
 * persistent trace launch over all rays in which every lane looks up its
 * ray's mesh.  Each mesh's tree, index buffer and hits are bit-identical to
 * rta_lbvh_build + rta_trace of that mesh alone (its triangle ids and hit
 * refs are local to the mesh).  No counterpart in the reference, which builds
 * one mesh per lbvh_constructor (lbvh.h:153-211). */
typedef struct rta_batch rta_batch;

/* Launch parameters of a batch (chosen by rta_batch_autotune or set). */
typedef struct rta_batch_params {
    int digit_bits;     /* sort digit width: 8, 9, 10 or 11 */
    int fetch_idle;     /* a warp fetches rays once this many lanes are idle: 1..32 */
    int blocks_per_sm;  /* persistent trace blocks per SM, 0 = occupancy maximum */
    int stack;          /* traversal stack entries: 40 or 64 */
} rta_batch_params;

int rta_batch_create(rta_batch **out);
int rta_batch_destroy(rta_batch *b);

/* Declares the meshes and sizes the device buffers.  tri_offsets and
 * ray_offsets are HOST prefix arrays of meshes + 1 entries: mesh m owns
 * triangles [tri_offsets[m], tri_offsets[m+1]) of the concatenated input
 * (1 .. rta_lbvh_max_triangles() of them) and rays [ray_offsets[m],
 * ray_offsets[m+1]) (possibly none).  At most 2^20 meshes. */
int rta_batch_set_meshes(rta_batch *b, uint32_t meshes, const uint32_t *tri_offsets,
                         const uint32_t *ray_offsets);

/* Builds every mesh's LBVH from the concatenated 104-byte records (device). */
int rta_batch_build(rta_batch *b, const void *tris, rta_stream_t stream);

/* Closest-hit (child-is) trace of every mesh's rays against its own tree:
 * rays in the rta_trace layout, concatenated in mesh order; hits (16 bytes
 * per ray, t = FLT_MAX on entry as rta_reset_intersections leaves it) are
 * written in the same order; stats as in rta_trace (nullable). */
int rta_batch_trace(rta_batch *b, const float *orig, const float *dir, const float *maxt, void *hits,
                    uint32_t *stats, rta_stream_t stream);

/* Build + hit reset (as rta_reset_intersections) + trace as one CUDA graph launch.  The graph is captured
 * on the first call and again whenever the pointers or the parameters
 * change; the call that captures also launches it. */
int rta_batch_run(rta_batch *b, const void *tris, const float *orig, const float *dir,
                  const float *maxt, void *hits, rta_stream_t stream);

/* The tree of one mesh as a one-mesh view (for rta_trace, rta_lbvh_to_2f4
 * and the parity checks).  Valid until the next set_meshes / destroy. */
int rta_batch_mesh(const rta_batch *b, uint32_t mesh, rta_lbvh *out);

/* Device flags of the last build / trace (RTA_DEV_*); synchronises stream. */
int rta_batch_status(const rta_batch *b, rta_stream_t stream, uint32_t *flags);

int rta_batch_get_params(const rta_batch *b, rta_batch_params *p);
int rta_batch_set_params(rta_batch *b, const rta_batch_params *p);

/* Autotuner: times rta_batch_run (median of reps graph launches) while it
 * walks the parameters one at a time over their candidate values (digit
 * width, fetch threshold, blocks per SM, stack), keeps the fastest and sets
 * it.  With a cache_path (nullable), a cached choice for this device and
 * workload is used without timing, and a new choice is stored there. */
int rta_batch_autotune(rta_batch *b, const void *tris, const float *orig, const float *dir,
                       const float *maxt, void *hits, const char *cache_path, int reps,
                       rta_stream_t stream, rta_batch_params *chosen, float *best_ms);

/* The autotuner's cache key of b (device name, SM count, mesh count and the
 * power-of-two classes of the triangle and ray counts). */
int rta_batch_tune_key(const rta_batch *b, char *buf, uint32_t size);

/* The tuning cache: a JSON object, one entry per line, key -> parameters and
 * time.  Work without a device.  lookup returns RTA_ERR_INVALID when the
 * file or the key is absent. */
int rta_tune_cache_lookup(const char *path, const char *key, rta_batch_params *p);
int rta_tune_cache_store(const char *path, const char *key, const rta_batch_params *p, float ms);

#ifdef __cplusplus
}
#endif
#endif
