// trace.cu -- binary-BVH traversal on sm_103a.
//
// Persistent warps pull rays from a global atomic queue; each lane traverses
// one ray with a short stack in local memory (L1-resident), and idle lanes
// refill from the queue while the rest of the warp is still busy.
// The arithmetic is the reference's, operation for operation, through
// explicit round-to-nearest intrinsics so no multiply-add is ever fused:
//   slab test        intersect_aabb          (librta/intersect.h:56-150)
//   Aila box test    intersect_aabb_aila     (librta/intersect.h:165-176)
//   triangle test    intersect_tri_opt       (librta/intersect.h:8-53)
// and the visiting order is that of the 2F4 kernels
//   CIS  trace_cis(float4*)  (bbvh-cuda/kernels.cu:777-855)
//   DIS  trace_dis(float4*)  (bbvh-cuda/kernels.cu:486-548)
// so hits, including which of two equal-t triangles wins, are the reference's.
#include "common.cuh"
#include "batch.cuh"
#include "bounce.cuh"
#include "mlp.cuh"

namespace rta {

struct TraceArgs {
    const NodeRec *nodes;
    const RootRec *root;
    const TriRec *tris;
    const float *orig, *dir, *maxt;
    uint32_t nrays;
    const uint32_t *d_nrays;
    HitRec *hits;
    uint32_t *stats;
    uint32_t *queue;    // ray batch counter, zero at launch
    uint32_t *status;
    uint32_t n_tris;    // bounds every link and triangle index before use
    // FUSE (frame with one diffuse bounce): each primary hit's bounce ray is
    // traced by the same lane right after it; its ray and hit go to the
    // primary ray's slot, flagged, for the ordered compaction that follows
    uint32_t seed;
    float eps;
    float *b_orig, *b_dir;
    HitRec *b_hits;
    uint32_t *b_flag;
    uint32_t *b_tile;   // bounce rays per 2^kBounceTileLog2 primary rays (zero at launch)
};

// three-input min / max (sm_100 family); NaN inputs are ignored as by fminf / fmaxf
__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Per-ray constants of the slab test: the ray, which direction components
// are zero (intersect_aabb treats d == 0 separately) and the constants of the
// division-free filter below.
struct Ray {
    float o[3], d[3];
    uint32_t zero;   // bit k: d[k] == 0
    float tmax;
    float tmax_up;   // least float above tmax (+inf for a NaN tmax): t > tmax <=> t >= tmax_up
    float eabs;      // absolute error term of the filter's quotients, max |o[k] rd[k]| 2^-23 (+ 2^-146)
    bool fast;       // the filter applies: every |d[k]| in [2^-100, 2^100], o[k] rd[k] finite
    float rd[3];     // RN(1 / d[k]); the filter's quotients are fma(plane, rd[k], nord[k])
    float nord[3];   // -RN(o[k] rd[k])
};

__device__ __forceinline__ void make_ray(Ray &R, const float o[3], const float d[3], float tmax)
{
    R.zero = 0;
    bool fast = true;
    float eabs = 1.12103877e-44f;   // 2^-146
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R.o[k] = o[k];
        R.d[k] = d[k];
        if (d[k] == 0.0f) R.zero |= 1u << k;
        const float ad = fabsf(d[k]);
        fast = fast && ad >= 7.8886091e-31f && ad <= 1.2676506e30f;   // also false for 0, NaN, inf
        const float rd = d[k] == 0.0f ? 0.0f : __frcp_rn(d[k]);
        const float ord = __fmul_rn(o[k], rd);
        fast = fast && fabsf(ord) <= FLT_MAX;
        eabs = fmaxf(eabs, __fmaf_ru(fabsf(ord), 1.19209290e-07f, 1.12103877e-44f));
        R.rd[k] = rd;
        R.nord[k] = -ord;
    }
    R.tmax = tmax;
    // RU(tmax + 2^-149) is the next float up for every finite tmax (and +inf for +inf)
    R.tmax_up = tmax != tmax ? __int_as_float(0x7f800000) : (tmax < -FLT_MAX ? -FLT_MAX : __fadd_ru(tmax, 1.40129846e-45f));
    R.eabs = eabs;
    R.fast = fast;
}

// intersect_aabb (librta/intersect.h:56-150).  The reference walks the axes
// with early outs; t_near only grows and t_far only shrinks along the way, so
// "no early out fired" equals "t_near <= t_far and t_far >= 0 at the end and
// every zero-direction axis has the origin inside the slab".  The quotients
// are the reference's correctly rounded (lo - o) / d.
__device__ __forceinline__ bool slab_test(float lx, float hx, float ly, float hy, float lz, float hz,
                                          const Ray &R, float &dist, float &far)
{
    const float lo[3] = {lx, ly, lz}, hi[3] = {hx, hy, hz};
    float t_near = -FLT_MAX, t_far = FLT_MAX;
    bool inside = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (R.zero & (1u << k)) {
            inside = inside && !(R.o[k] < lo[k] || R.o[k] > hi[k]);
        } else {
            float t1 = __fdiv_rn(__fsub_rn(lo[k], R.o[k]), R.d[k]);
            float t2 = __fdiv_rn(__fsub_rn(hi[k], R.o[k]), R.d[k]);
            t_near = fmaxf(t_near, fminf(t1, t2));
            t_far = fminf(t_far, fmaxf(t1, t2));
        }
    }
    dist = t_near;
    far = t_far;
    return inside && t_near <= t_far && t_far >= 0.0f;
}

__device__ __forceinline__ bool slab_test(float lx, float hx, float ly, float hy, float lz, float hz,
                                          const Ray &R, float &dist)
{
    float far;
    return slab_test(lx, hx, ly, hy, lz, hz, R, dist, far);
}

// ---- exact slab decisions without divisions, where they are certain ----
//
// The child-is step needs only decisions from the slab test: does each child
// count as hit (inside, t_near <= t_far, t_far >= 0, and not culled:
// t_near < best t, t_near <= t_max), and is the left t_near <= the right one.
// With r = RN(1/d) and the fused quotient q = RN(plane * r - RN(o * r)) (one
// FMA per plane), q is within |q| * 2^-21 + |o r| * 2^-23 of the reference's
// RN(RN(plane - o) / d): relative roundings of 2^-24 for r, for o * r, for
// the FMA, for plane - o and for the reference's division, plus the
// cancellation term of o * r; 2^-146 absolute covers subnormal results.
// t_near is a max and t_far a min of such quotients, so the exact t_near /
// t_far lie within |t| * 2^-21 + max_k |o_k r_k| * 2^-23 + 2^-146 of the
// approximate ones (the bound of the quotient that attains the max or min
// dominates every other's; the absolute term is one per ray).  The bounds
// are rounded outward.  A decision is taken from the intervals when it is the
// same for every value in them; otherwise the step falls back to the exact
// divisions.  NaN bounds (overflowing quotients) always count as uncertain.
// The filter applies to rays without a zero direction component and with
// finite o * r (R.fast); the others take the exact test at every step.  On
// the 1080p terrain frame the exact fallback runs in 0.03 % of the child-is
// steps (0.5 % of warp iterations).
#ifndef RTA_SLAB_FILTER
#define RTA_SLAB_FILTER 1
#endif
constexpr float kFilterRel = 4.76837158e-07f;   // 2^-21
constexpr float kFilterAbs = 1.12103877e-44f;   // 2^-146

// The decision from outward-rounded bounds of t_near and t_far.  cull =
// min(best t, tmax_up): "t_near >= best t or t_near > tmax" is t_near >= cull.
// 0: certainly not a kept hit; 1: certainly a kept hit; 2: uncertain.
// [lo, hi] bounds the exact t_near when the child is kept.
__device__ __forceinline__ int filter_bounds(float tn_lo, float tn_hi, float tf_lo, float tf_hi, float cull,
                                             float &lo, float &hi)
{
    // hit = t_near <= t_far && t_far >= 0; kept = hit && t_near < cull
    if (tn_lo > tf_hi || tf_hi < 0.0f || tn_lo >= cull) return 0;   // certainly not
    lo = tn_lo;
    hi = tn_hi;
    if (tn_hi <= tf_lo && tf_lo >= 0.0f && tn_hi < cull) return 1;   // certainly
    return 2;
}

// One box; R.fast is a precondition (no zero direction component).  t_near
// and t_far as max / min over the axes need no -FLT_MAX / FLT_MAX start: a
// quotient of +-inf (overflow) makes the bounds inf or NaN, which decide
// nothing certain unless the other, finite, distance does.
__device__ __forceinline__ int slab_filter(float lx, float hx, float ly, float hy, float lz, float hz,
                                           const Ray &R, float cull, float &lo, float &hi)
{
    const float qlx = __fmaf_rn(lx, R.rd[0], R.nord[0]), qhx = __fmaf_rn(hx, R.rd[0], R.nord[0]);
    const float qly = __fmaf_rn(ly, R.rd[1], R.nord[1]), qhy = __fmaf_rn(hy, R.rd[1], R.nord[1]);
    const float qlz = __fmaf_rn(lz, R.rd[2], R.nord[2]), qhz = __fmaf_rn(hz, R.rd[2], R.nord[2]);
    const float tn = max3f(fminf(qlx, qhx), fminf(qly, qhy), fminf(qlz, qhz));
    const float tf = min3f(fmaxf(qlx, qhx), fmaxf(qly, qhy), fmaxf(qlz, qhz));
    const float wn = __fmaf_ru(fabsf(tn), kFilterRel, R.eabs);
    const float wf = __fmaf_ru(fabsf(tf), kFilterRel, R.eabs);
    return filter_bounds(__fsub_rd(tn, wn), __fadd_ru(tn, wn), __fsub_rd(tf, wf), __fadd_ru(tf, wf), cull, lo,
                         hi);
}

// The entry distance of one box from its near planes: the approximate
// quotient of every axis, the axis that attains the max, and whether that
// axis certainly attains the exact max too (every other axis' exact quotient
// is certainly smaller).  Then the exact entry distance is
// RN((plane - o) / d) of that one axis; `num` is its numerator plane - o and
// `den` its d.  (Selects, not indexing: a run-time index would put the ray
// into local memory.)
__device__ __forceinline__ bool entry_axis(float lx, float hx, float ly, float hy, float lz, float hz,
                                           const Ray &R, int &axis, float &plane, float &num, float &den)
{
    const float c0 = R.d[0] > 0.0f ? lx : hx, c1 = R.d[1] > 0.0f ? ly : hy, c2 = R.d[2] > 0.0f ? lz : hz;
    const float a0 = __fsub_rn(c0, R.o[0]), a1 = __fsub_rn(c1, R.o[1]), a2 = __fsub_rn(c2, R.o[2]);
    const float q0 = __fmul_rn(a0, R.rd[0]);
    const float q1 = __fmul_rn(a1, R.rd[1]);
    const float q2 = __fmul_rn(a2, R.rd[2]);
    const bool k2 = q2 >= fmaxf(q0, q1);
    const bool k1 = !k2 && q1 >= q0;
    const float top = k2 ? q2 : (k1 ? q1 : q0);
    const float second = k2 ? fmaxf(q0, q1) : (k1 ? fmaxf(q0, q2) : fmaxf(q1, q2));
    axis = k2 ? 2 : (k1 ? 1 : 0);
    plane = k2 ? c2 : (k1 ? c1 : c0);
    num = k2 ? a2 : (k1 ? a1 : a0);
    den = k2 ? R.d[2] : (k1 ? R.d[1] : R.d[0]);
    const float wt = __fmaf_ru(fabsf(top), kFilterRel, kFilterAbs);
    const float ws = __fmaf_ru(fabsf(second), kFilterRel, kFilterAbs);
    return __fadd_ru(second, ws) < __fsub_rd(top, wt);
}

// dl <= dr for two kept children whose entry intervals overlap: equal planes
// give equal quotients (the reference then goes left); otherwise one exact
// division per child.  Returns false when an entry axis is not certain.
__device__ __forceinline__ bool order_resolve(const NodeRec &nd, const Ray &R, bool &left_first)
{
    int kl, kr;
    float cl, cr, nl, nr, dl_den, dr_den;
    if (!entry_axis(RTA_LEFT_BOX(nd), R, kl, cl, nl, dl_den)) return false;
    if (!entry_axis(RTA_RIGHT_BOX(nd), R, kr, cr, nr, dr_den)) return false;
    if (kl == kr && __float_as_uint(cl) == __float_as_uint(cr)) {
        left_first = true;
        return true;
    }
    left_first = __fdiv_rn(nl, dl_den) <= __fdiv_rn(nr, dr_den);
    return true;
}

// Outward-rounded bounds of one box's t_near and t_far from the approximate
// quotients (R.fast is a precondition).
__device__ __forceinline__ void slab_bounds(float lx, float hx, float ly, float hy, float lz, float hz,
                                            const Ray &R, float &tn_lo, float &tn_hi, float &tf_lo, float &tf_hi)
{
    const float qlx = __fmaf_rn(lx, R.rd[0], R.nord[0]), qhx = __fmaf_rn(hx, R.rd[0], R.nord[0]);
    const float qly = __fmaf_rn(ly, R.rd[1], R.nord[1]), qhy = __fmaf_rn(hy, R.rd[1], R.nord[1]);
    const float qlz = __fmaf_rn(lz, R.rd[2], R.nord[2]), qhz = __fmaf_rn(hz, R.rd[2], R.nord[2]);
    const float tn = max3f(fminf(qlx, qhx), fminf(qly, qhy), fminf(qlz, qhz));
    const float tf = min3f(fmaxf(qlx, qhx), fmaxf(qly, qhy), fmaxf(qlz, qhz));
    const float wn = __fmaf_ru(fabsf(tn), kFilterRel, R.eabs);
    const float wf = __fmaf_ru(fabsf(tf), kFilterRel, R.eabs);
    tn_lo = __fsub_rd(tn, wn);
    tn_hi = __fadd_ru(tn, wn);
    tf_lo = __fsub_rd(tf, wf);
    tf_hi = __fadd_ru(tf, wf);
}

// The child-is decisions of one node: hl / hr (child hit and not culled) and
// left_first, the child to visit first among the kept ones (dl <= dr when
// both are kept); exact, through the filter where it is certain.  The
// filter's "certainly kept" and "certainly not" are predicates, never both
// true (certainly kept implies tn_lo <= tn_hi <= tf_lo <= tf_hi, tf_lo >= 0
// and tn_lo <= tn_hi < cull).
__device__ __forceinline__ void cis_decide(const NodeRec &nd, const Ray &R, float best_t, bool &hl, bool &hr,
                                           bool &left_first)
{
    if (RTA_SLAB_FILTER && R.fast) {
        const float cull = fminf(best_t, R.tmax_up);
        float lnl, lnh, lfl, lfh, rnl, rnh, rfl, rfh;
        slab_bounds(RTA_LEFT_BOX(nd), R, lnl, lnh, lfl, lfh);
        slab_bounds(RTA_RIGHT_BOX(nd), R, rnl, rnh, rfl, rfh);
        // hit = t_near <= t_far && t_far >= 0; kept = hit && t_near < cull
        const bool l_yes = lnh <= lfl && lfl >= 0.0f && lnh < cull;
        const bool r_yes = rnh <= rfl && rfl >= 0.0f && rnh < cull;
        const bool l_no = lnl > lfh || lfh < 0.0f || lnl >= cull;
        const bool r_no = rnl > rfh || rfh < 0.0f || rnl >= cull;
        if ((l_yes || l_no) && (r_yes || r_no)) {
            hl = l_yes;
            hr = r_yes;
            // both kept: the entry intervals order them, else the exact entry
            left_first = l_yes && (!r_yes || lnh <= rnl);
            if (!(l_yes && r_yes) || lnh <= rnl || lnl > rnh) return;
            if (order_resolve(nd, R, left_first)) return;
        }
    }
    float dl = FLT_MAX, dr = FLT_MAX;
    hl = slab_test(RTA_LEFT_BOX(nd), R, dl);
    hr = slab_test(RTA_RIGHT_BOX(nd), R, dr);
    if (dl >= best_t || dl > R.tmax) hl = false;
    if (dr >= best_t || dr > R.tmax) hr = false;
    left_first = hl && (!hr || dl <= dr);
}

// intersect_aabb_aila with the ailabox kernels' reciprocal (kernels.cu:966-970)
__device__ __forceinline__ bool aila_test(float lx, float hx, float ly, float hy, float lz, float hz,
                                          const float o[3], const float id[3], float t, float &ret)
{
    const float lo[3] = {lx, ly, lz}, hi[3] = {hx, hy, hz};
    float t1[3], t2[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float oid = __fmul_rn(o[k], id[k]);
        t1[k] = __fsub_rn(__fmul_rn(lo[k], id[k]), oid);
        t2[k] = __fsub_rn(__fmul_rn(hi[k], id[k]), oid);
    }
    float near = fmaxf(fmaxf(fminf(t1[0], t2[0]), fminf(t1[1], t2[1])), fminf(t1[2], t2[2]));
    float far = fminf(fminf(fmaxf(t1[0], t2[0]), fmaxf(t1[1], t2[1])), fmaxf(t1[2], t2[2]));
    ret = near;
    return near <= far && far >= 0.f && near < t;
}

// intersect_tri_opt, expression for expression.  A quotient x/M can only be
// > 0 when x and M are non-zero with equal signs, so the three divisions are
// skipped when that already fails (the result is a miss either way).
__device__ __forceinline__ bool tri_test(const TriRec &T, const float o[3], const float dir[3],
                                         float &tt_out, float &beta_out, float &gamma_out)
{
    const float a_x = T.v0.x, a_y = T.v0.y, a_z = T.v0.z;
    const float a = __fsub_rn(a_x, T.v1.x);
    const float b = __fsub_rn(a_y, T.v1.y);
    const float c = __fsub_rn(a_z, T.v1.z);
    const float d = __fsub_rn(a_x, T.v2.x);
    const float e = __fsub_rn(a_y, T.v2.y);
    const float f = __fsub_rn(a_z, T.v2.z);
    const float g = dir[0], h = dir[1], i = dir[2];
    const float j = __fsub_rn(a_x, o[0]);
    const float k = __fsub_rn(a_y, o[1]);
    const float l = __fsub_rn(a_z, o[2]);
    float common1 = __fsub_rn(__fmul_rn(e, i), __fmul_rn(h, f));
    float common2 = __fsub_rn(__fmul_rn(g, f), __fmul_rn(d, i));
    float common3 = __fsub_rn(__fmul_rn(d, h), __fmul_rn(e, g));
    float M = __fadd_rn(__fadd_rn(__fmul_rn(a, common1), __fmul_rn(b, common2)), __fmul_rn(c, common3));
    float beta = __fadd_rn(__fadd_rn(__fmul_rn(j, common1), __fmul_rn(k, common2)), __fmul_rn(l, common3));
    common1 = __fsub_rn(__fmul_rn(a, k), __fmul_rn(j, b));
    common2 = __fsub_rn(__fmul_rn(j, c), __fmul_rn(a, l));
    common3 = __fsub_rn(__fmul_rn(b, l), __fmul_rn(k, c));
    float gamma = __fadd_rn(__fadd_rn(__fmul_rn(i, common1), __fmul_rn(h, common2)), __fmul_rn(g, common3));
    float tt = -__fadd_rn(__fadd_rn(__fmul_rn(f, common1), __fmul_rn(e, common2)), __fmul_rn(d, common3));
    const uint32_t sm = __float_as_uint(M) >> 31;
    if (M == 0.0f || tt == 0.0f || beta == 0.0f || gamma == 0.0f ||
        (__float_as_uint(tt) >> 31) != sm || (__float_as_uint(beta) >> 31) != sm ||
        (__float_as_uint(gamma) >> 31) != sm)
        return false;
    beta = __fdiv_rn(beta, M);
    gamma = __fdiv_rn(gamma, M);
    tt = __fdiv_rn(tt, M);
    if (tt > 0.0f && beta > 0.0f && gamma > 0.0f && __fadd_rn(beta, gamma) <= 1.0f) {
        tt_out = tt;
        beta_out = beta;
        gamma_out = gamma;
        return true;
    }
    return false;
}

__device__ __forceinline__ NodeRec load_node(const NodeRec *nodes, uint32_t idx)
{
    const float4 *p = reinterpret_cast<const float4 *>(nodes + idx);
    NodeRec r;
    r.q0 = __ldg(p + 0);
    r.q1 = __ldg(p + 1);
    r.q2 = __ldg(p + 2);
    float4 q3 = __ldg(p + 3);
    r.q3 = make_uint4(__float_as_uint(q3.x), __float_as_uint(q3.y), __float_as_uint(q3.z),
                      __float_as_uint(q3.w));
    return r;
}

__device__ __forceinline__ TriRec load_tri(const TriRec *tris, uint32_t idx)
{
    const float4 *p = reinterpret_cast<const float4 *>(tris + idx);
    TriRec t;
    t.v0 = __ldg(p + 0);
    t.v1 = __ldg(p + 1);
    t.v2 = __ldg(p + 2);
    return t;
}

// no ray visits more nodes than this; a corrupt tree ends the ray with a flag
constexpr uint32_t kMaxSteps = 1u << 22;
constexpr int kTraceThreads = 128;
// idle lanes of a warp fetch new rays once at least this many are idle
#ifndef RTA_FETCH_IDLE
#define RTA_FETCH_IDLE 12
#endif
constexpr int kFetchIdle = RTA_FETCH_IDLE;
// LEARNED: a network pass runs once this many lanes of a warp wait for a
// decision (or every active lane does)
#ifndef RTA_PARK_MIN
#define RTA_PARK_MIN 16
#endif
constexpr int kParkMin = RTA_PARK_MIN;

struct Best {
    float t, beta, gamma;
    uint32_t ref;
};

// tests the triangles of one leaf; returns true if a shadow ray may stop
template <bool SHADOW>
__device__ __forceinline__ bool visit_leaf(const TriRec *tris, uint32_t n_tris, uint32_t link,
                                           const float o[3], const float d[3], float tmax, Best &best,
                                           uint32_t &tri_tests, bool &bad)
{
    const uint32_t first = leaf_first(link);
    if (first >= n_tris) { bad = true; return true; }
    TriRec t0 = load_tri(tris, first);
    uint32_t f = leaf_count_field(link);
    uint32_t count = f < 63u ? f + 1u : __float_as_uint(t0.v0.w);
    if (count > n_tris - first) { bad = true; return true; }
    for (uint32_t i = 0; i < count; ++i) {
        TriRec T = i ? load_tri(tris, first + i) : t0;
        ++tri_tests;
        float t, b, g;
        if (tri_test(T, o, d, t, b, g)) {
            if (t < best.t && t <= tmax) {
                best.t = t;
                best.beta = b;
                best.gamma = g;
                best.ref = first + i;
                if (SHADOW) break;
            }
        }
    }
    return SHADOW && best.t != FLT_MAX;
}

// One lane = one ray at a time; each loop iteration visits one node.  Lanes
// whose ray has finished take new rays from the global queue as soon as
// kFetchIdle of them are idle, so warps stay full while the queue lasts.
// RTA_SMEM_STACK: the traversal stack of k_trace lives in shared memory, one
// column per thread (entry i of thread t at i * threads + t: no bank
// conflicts), instead of per-thread local memory, for stacks of up to 48
// (1.4 % off the 1080p frame: the stack no longer competes with node
// fetches for L1)
#ifndef RTA_SMEM_STACK
#define RTA_SMEM_STACK 1
#endif

template <int STACK, bool SMEM> struct TraceStack;
template <int STACK> struct TraceStack<STACK, false> {
    uint32_t v[STACK];
    __device__ __forceinline__ void init(uint32_t *) {}
    __device__ __forceinline__ uint32_t &operator[](int i) { return v[i]; }
};
template <int STACK> struct TraceStack<STACK, true> {
    uint32_t *base;
    __device__ __forceinline__ void init(uint32_t *s) { base = s + threadIdx.x; }
    __device__ __forceinline__ uint32_t &operator[](int i) { return base[i * kTraceThreads]; }
};

// a lane at a leaf waits for this many leaf lanes before testing (0: never
// waits); 4 measured best on the 1080p terrain frame (2 %, sweep 2-16)
#ifndef RTA_LEAF_PARK
#define RTA_LEAF_PARK 4
#endif

// blocks per SM the compiler must fit in registers for the child-is kernels
// (8 = 64 registers: full occupancy beats the few spilled bytes, 3 % on the
// 1080p frame; the direct-is / Aila kernels keep their register count)
#ifndef RTA_TRACE_MIN_BLOCKS
#define RTA_TRACE_MIN_BLOCKS 8
#endif

template <bool DIS, bool SHADOW, bool AILA, bool STATS, int STACK, bool FUSE = false>
__global__ void __launch_bounds__(kTraceThreads, (!DIS && !AILA) ? RTA_TRACE_MIN_BLOCKS : 0) k_trace(TraceArgs A)
{
    static_assert(!FUSE || (!DIS && !SHADOW && !AILA && !STATS), "the fused frame is child-is closest hit");
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t nrays = A.d_nrays ? *A.d_nrays : A.nrays;
    const RootRec root = *A.root;
    const uint32_t n_inner = A.n_tris - 1u;

    bool active = false, exhausted = false;
    uint32_t r = 0, cur = 0, steps = 0, inner_visits = 0, tri_tests = 0;
    int sp = -1;
    constexpr bool kSmemStack = RTA_SMEM_STACK && STACK <= 48;
    __shared__ uint32_t s_stack[kSmemStack ? STACK * kTraceThreads : 1];
    TraceStack<STACK, kSmemStack> stack;
    stack.init(s_stack);
    Ray R;
    float id[3] = {0.f, 0.f, 0.f};
    Best best;
    float bx[6];   // DIS: box of the current node
    bool overflow = false, capped = false, bad = false;
    bool second = false;    // FUSE: the lane traces ray r's bounce ray
    bool pending = false;   // FUSE: ray r hit; its bounce ray is made at the next fetch

    for (;;) {
        // idle lanes (pending ones included) take new rays together once
        // kFetchIdle of them are idle: a pending lane its own bounce ray, the
        // others rays from the queue.  The branch is warp-uniform.
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        const uint32_t pend = FUSE ? __ballot_sync(0xffffffffu, pending) : 0u;
        if ((__popc(idle) >= kFetchIdle && (!exhausted || pend != 0u)) || (pend != 0u && idle == 0xffffffffu)) {
            const uint32_t want = idle & ~pend;
            bool queued = false;
            uint32_t base = 0;
            if (!exhausted && want != 0u) {
                const int leader = __ffs(want) - 1;
                if ((int)lane == leader) base = atomicAdd(A.queue, (uint32_t)__popc(want));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (base >= nrays) exhausted = true;
                else queued = true;
            }
            if (!active) {
                float o[3], d[3], tmax = FLT_MAX;
                bool got = false;
                if (FUSE && pending) {
                    // the bounce ray of ray r's hit (bounce.cuh)
                    bounce_ray(load_tri(A.tris, best.ref), R.o, R.d, best.t, r, A.seed, A.eps, o, d);
                    A.b_orig[3 * (size_t)r + 0] = o[0];
                    A.b_orig[3 * (size_t)r + 1] = o[1];
                    A.b_orig[3 * (size_t)r + 2] = o[2];
                    A.b_dir[3 * (size_t)r + 0] = d[0];
                    A.b_dir[3 * (size_t)r + 1] = d[1];
                    A.b_dir[3 * (size_t)r + 2] = d[2];
                    pending = false;
                    second = true;
                    got = true;
                } else if (queued) {
                    r = base + __popc(want & lt_mask);
                    if (r < nrays) {
                        o[0] = A.orig[3 * (size_t)r + 0];
                        o[1] = A.orig[3 * (size_t)r + 1];
                        o[2] = A.orig[3 * (size_t)r + 2];
                        d[0] = A.dir[3 * (size_t)r + 0];
                        d[1] = A.dir[3 * (size_t)r + 1];
                        d[2] = A.dir[3 * (size_t)r + 2];
                        tmax = A.maxt[r];
                        second = false;
                        got = true;
                    }
                }
                if (got) {
                    make_ray(R, o, d, tmax);
                    if (AILA) {
                        const float ooeps = 8.27180612553027674871e-25f;   // exp2f(-80)
#pragma unroll
                        for (int k = 0; k < 3; ++k)
                            id[k] = __fdiv_rn(1.0f, fabsf(d[k]) > ooeps ? d[k] : copysignf(ooeps, d[k]));
                    }
                    best.t = FLT_MAX;
                    best.beta = best.gamma = 0.f;
                    best.ref = 0;
                    sp = -1;
                    steps = inner_visits = tri_tests = 0;
                    cur = root.link;
                    if (DIS) {
                        bx[0] = root.lo[0]; bx[1] = root.hi[0]; bx[2] = root.lo[1];
                        bx[3] = root.hi[1]; bx[4] = root.lo[2]; bx[5] = root.hi[2];
                    }
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (!DIS && RTA_LEAF_PARK > 0) {
            // a lane at a leaf waits until enough lanes of the warp are at
            // leaves (or every active lane is), so the warp runs the triangle
            // tests together instead of beside inner-node steps; each ray
            // still visits its nodes in the same order
            const bool at_leaf = active && is_leaf(cur);
            const uint32_t lm = __ballot_sync(0xffffffffu, at_leaf);
            const uint32_t am = __ballot_sync(0xffffffffu, active);
            if (at_leaf && __popc(lm) < RTA_LEAF_PARK && lm != am) continue;
        }
        if (!active) continue;

        // ---- one traversal step ----
        bool done = false;
        ++steps;
        if (!DIS) {
            // child-is (kernels.cu:797-852): test both children, nearer first.
            // A broken link and a runaway ray share one rare branch; only
            // inner steps push, so capping them bounds every ray.
            if (!is_leaf(cur)) {
                if (cur >= n_inner || steps > kMaxSteps) {
                    bad = bad || cur >= n_inner;
                    capped = capped || cur < n_inner;
                    done = true;
                } else {
                    ++inner_visits;
                    const NodeRec nd = load_node(A.nodes, cur);
                    bool hl, hr, left_first;
                    if (AILA) {
                        float dl = FLT_MAX, dr = FLT_MAX;
                        hl = aila_test(RTA_LEFT_BOX(nd), R.o, id, best.t, dl);
                        hr = aila_test(RTA_RIGHT_BOX(nd), R.o, id, best.t, dr);
                        if (dl >= best.t || dl > R.tmax) hl = false;
                        if (dr >= best.t || dr > R.tmax) hr = false;
                        left_first = hl && (!hr || dl <= dr);
                    } else {
                        cis_decide(nd, R, best.t, hl, hr, left_first);
                    }
                    if (hl || hr) {
                        // the first kept child next; with both kept the other one onto the stack
                        cur = left_first ? nd.q3.x : nd.q3.y;
                        if (hl && hr) {
                            if (sp + 1 >= STACK) {
                                overflow = true;
                                done = true;
                            } else {
                                stack[++sp] = left_first ? nd.q3.y : nd.q3.x;
                            }
                        }
                    } else if (sp < 0) {
                        done = true;
                    } else {
                        cur = stack[sp--];
                    }
                }
            } else {
                if (visit_leaf<SHADOW>(A.tris, A.n_tris, cur, R.o, R.d, R.tmax, best, tri_tests, bad))
                    done = true;
                else if (sp < 0)
                    done = true;
                else
                    cur = stack[sp--];
            }
        } else if (steps > kMaxSteps) {
            capped = true;
            done = true;
        } else {
            // direct-is (kernels.cu:506-545): a node's own box is tested when it
            // is visited; the stack holds (parent << 1 | side) and a popped
            // node's box is re-read from its parent's record
            bool pop = false;
            if (!is_leaf(cur)) {
                ++inner_visits;
                bool h;
                int certain = 2;
                if (!AILA && RTA_SLAB_FILTER && R.fast) {
                    float lo, hi;
                    certain = slab_filter(bx[0], bx[1], bx[2], bx[3], bx[4], bx[5], R, fminf(best.t, R.tmax_up), lo,
                                          hi);
                }
                if (certain != 2) {
                    h = certain == 1;
                } else {
                    float dist = FLT_MAX;
                    h = AILA ? aila_test(bx[0], bx[1], bx[2], bx[3], bx[4], bx[5], R.o, id, best.t, dist)
                             : slab_test(bx[0], bx[1], bx[2], bx[3], bx[4], bx[5], R, dist);
                    if (dist >= best.t || dist > R.tmax) h = false;
                }
                if (h) {
                    if (sp + 1 >= STACK) {
                        overflow = true;
                        done = true;
                    } else if (cur >= n_inner) {
                        bad = true;
                        done = true;
                    } else {
                        const NodeRec nd = load_node(A.nodes, cur);
                        stack[++sp] = (cur << 1) | 1u;
                        cur = nd.q3.x;
                        bx[0] = nd.q0.x; bx[1] = nd.q0.z; bx[2] = nd.q1.x;
                        bx[3] = nd.q1.z; bx[4] = nd.q2.x; bx[5] = nd.q2.z;
                    }
                } else {
                    pop = true;
                }
            } else {
                if (visit_leaf<SHADOW>(A.tris, A.n_tris, cur, R.o, R.d, R.tmax, best, tri_tests, bad))
                    done = true;
                else
                    pop = true;
            }
            if (pop && !done) {
                if (sp < 0) {
                    done = true;
                } else {
                    const uint32_t e = stack[sp--];
                    if ((e >> 1) >= n_inner) {
                        bad = true;
                        done = true;
                    } else {
                        const NodeRec nd = load_node(A.nodes, e >> 1);
                        if (e & 1u) {
                            cur = nd.q3.y;
                            bx[0] = nd.q0.y; bx[1] = nd.q0.w; bx[2] = nd.q1.y;
                            bx[3] = nd.q1.w; bx[4] = nd.q2.y; bx[5] = nd.q2.w;
                        } else {
                            cur = nd.q3.x;
                            bx[0] = nd.q0.x; bx[1] = nd.q0.z; bx[2] = nd.q1.x;
                            bx[3] = nd.q1.z; bx[4] = nd.q2.x; bx[5] = nd.q2.z;
                        }
                    }
                }
            }
        }
        if (done) {
            if (FUSE) {
                // a miss leaves the record as the frame's reset left it:
                // t = FLT_MAX, beta = 1, gamma = 2 (reset_intersections), ref kept
                HitRec *out = second ? A.b_hits : A.hits;
                if (best.t != FLT_MAX) {
                    reinterpret_cast<float4 *>(out)[r] =
                        make_float4(best.t, best.beta, best.gamma, __uint_as_float(best.ref));
                } else {
                    out[r].t = FLT_MAX;
                    out[r].beta = 1.0f;
                    out[r].gamma = 2.0f;
                }
                const bool bounce = !second && best.t != FLT_MAX && best.ref < A.n_tris;
                if (!second) A.b_flag[r] = bounce ? 1u : 0u;
                if (bounce) atomicAdd(A.b_tile + (r >> kBounceTileLog2), 1u);
                pending = bounce;
                active = false;
            } else {
                if (best.t != FLT_MAX) {
                    reinterpret_cast<float4 *>(A.hits)[r] =
                        make_float4(best.t, best.beta, best.gamma, __uint_as_float(best.ref));
                } else {
                    A.hits[r].t = FLT_MAX;
                }
                if (STATS) {
                    A.stats[2 * (size_t)r + 0] = inner_visits;
                    A.stats[2 * (size_t)r + 1] = tri_tests;
                }
                active = false;
            }
        }
    }
    if (overflow) atomicOr(A.status, RTA_DEV_STACK_OVERFLOW);
    if (capped) atomicOr(A.status, RTA_DEV_ITER_LIMIT);
    if (bad) atomicOr(A.status, RTA_DEV_BAD_LINK);
}

// ------------------------------------------------------------------------- //
// batched child-is traversal: many meshes, one persistent launch             //
// ------------------------------------------------------------------------- //
//
// The step loop of k_trace<CIS> over the rays of all meshes of a batch.  A
// lane that takes ray r finds its mesh by a binary search over the rays'
// prefix offsets and from then on walks that mesh's tree (its own node,
// triangle and root pointers), so the warps stay full across mesh borders.
// fetch_idle is a launch parameter here (the autotuner sets it).

template <bool STATS, int STACK>
__global__ void __launch_bounds__(kTraceThreads) k_trace_batch(BatchTraceArgs A)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t nrays = A.nrays;

    bool active = false, exhausted = false;
    uint32_t r = 0, cur = 0, steps = 0, inner_visits = 0, tri_tests = 0;
    int sp = -1;
    constexpr bool kSmemStack = RTA_SMEM_STACK && STACK <= 48;
    __shared__ uint32_t s_stack[kSmemStack ? STACK * kTraceThreads : 1];
    TraceStack<STACK, kSmemStack> stack;
    stack.init(s_stack);
    Ray R;
    Best best;
    const NodeRec *nodes = nullptr;
    const TriRec *tris = nullptr;
    uint32_t n_tris = 1, n_inner = 0;
    bool overflow = false, capped = false, bad = false;

    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && __popc(idle) >= A.fetch_idle) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(A.queue, (uint32_t)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base >= nrays) {
                exhausted = true;
            } else if (!active) {
                r = base + __popc(idle & lt_mask);
                if (r < nrays) {
                    const uint32_t m = find_range(A.ray_off, A.n_meshes, r);
                    const MeshRec mr = A.meshes[m];
                    nodes = A.nodes + mr.node_off;
                    tris = A.tris + mr.tri_off;
                    n_tris = mr.n_tris;
                    n_inner = n_tris - 1u;
                    float o[3], d[3];
                    o[0] = A.orig[3 * (size_t)r + 0];
                    o[1] = A.orig[3 * (size_t)r + 1];
                    o[2] = A.orig[3 * (size_t)r + 2];
                    d[0] = A.dir[3 * (size_t)r + 0];
                    d[1] = A.dir[3 * (size_t)r + 1];
                    d[2] = A.dir[3 * (size_t)r + 2];
                    make_ray(R, o, d, A.maxt[r]);
                    best.t = FLT_MAX;
                    best.beta = best.gamma = 0.f;
                    best.ref = 0;
                    sp = -1;
                    steps = inner_visits = tri_tests = 0;
                    cur = A.roots[m].link;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (RTA_LEAF_PARK > 0) {   // leaf parking as in k_trace
            const bool at_leaf = active && is_leaf(cur);
            const uint32_t lm = __ballot_sync(0xffffffffu, at_leaf);
            const uint32_t am = __ballot_sync(0xffffffffu, active);
            if (at_leaf && __popc(lm) < RTA_LEAF_PARK && lm != am) continue;
        }
        if (!active) continue;

        bool done = false;
        ++steps;
        if (!is_leaf(cur)) {
            if (cur >= n_inner || steps > kMaxSteps) {   // as in k_trace
                bad = bad || cur >= n_inner;
                capped = capped || cur < n_inner;
                done = true;
            } else {
                ++inner_visits;
                const NodeRec nd = load_node(nodes, cur);
                bool hl, hr, left_first;
                cis_decide(nd, R, best.t, hl, hr, left_first);
                if (hl || hr) {
                    // the first kept child next; with both kept the other one onto the stack
                    cur = left_first ? nd.q3.x : nd.q3.y;
                    if (hl && hr) {
                        if (sp + 1 >= STACK) {
                            overflow = true;
                            done = true;
                        } else {
                            stack[++sp] = left_first ? nd.q3.y : nd.q3.x;
                        }
                    }
                } else if (sp < 0) {
                    done = true;
                } else {
                    cur = stack[sp--];
                }
            }
        } else {
            if (visit_leaf<false>(tris, n_tris, cur, R.o, R.d, R.tmax, best, tri_tests, bad))
                done = true;
            else if (sp < 0)
                done = true;
            else
                cur = stack[sp--];
        }
        if (done) {
            if (best.t != FLT_MAX) {
                reinterpret_cast<float4 *>(A.hits)[r] =
                    make_float4(best.t, best.beta, best.gamma, __uint_as_float(best.ref));
            } else {
                A.hits[r].t = FLT_MAX;
            }
            if (STATS) {
                A.stats[2 * (size_t)r + 0] = inner_visits;
                A.stats[2 * (size_t)r + 1] = tri_tests;
            }
            active = false;
        }
    }
    if (overflow) atomicOr(A.status, RTA_DEV_STACK_OVERFLOW);
    if (capped) atomicOr(A.status, RTA_DEV_ITER_LIMIT);
    if (bad) atomicOr(A.status, RTA_DEV_BAD_LINK);
}

// occupancy limit and SM count, queried once (before any graph capture:
// prepare_batch_trace() is called outside capture)
template <bool STATS, int STACK>
static void batch_grid(int &max_per_sm, int &sms)
{
    static int m = 0, n = 0;
    if (!m) {
        int dev = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_trace_batch<STATS, STACK>, kTraceThreads, 0);
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (m <= 0) m = 1;
        if (n <= 0) n = 1;
    }
    max_per_sm = m;
    sms = n;
}

template <bool STATS, int STACK>
static int launch_batch(const BatchTraceArgs &a, int blocks_per_sm, cudaStream_t s)
{
    int max_per_sm, sms;
    batch_grid<STATS, STACK>(max_per_sm, sms);
    const int per_sm = blocks_per_sm > 0 && blocks_per_sm < max_per_sm ? blocks_per_sm : max_per_sm;
    k_trace_batch<STATS, STACK><<<per_sm * sms, kTraceThreads, 0, s>>>(a);
    return check_launch("k_trace_batch");
}

int batch_trace_max_blocks_per_sm(int stack)
{
    int m, n;
    if (stack == 64) batch_grid<false, 64>(m, n);
    else batch_grid<false, 40>(m, n);
    batch_grid<true, 40>(m, n);
    batch_grid<true, 64>(m, n);
    if (stack == 64) batch_grid<false, 64>(m, n);
    else batch_grid<false, 40>(m, n);
    return m;
}

int launch_batch_trace(const BatchTraceArgs &a, int stack, int blocks_per_sm, cudaStream_t s)
{
    if (stack == 64)
        return a.stats ? launch_batch<true, 64>(a, blocks_per_sm, s) : launch_batch<false, 64>(a, blocks_per_sm, s);
    return a.stats ? launch_batch<true, 40>(a, blocks_per_sm, s) : launch_batch<false, 40>(a, blocks_per_sm, s);
}

// ------------------------------------------------------------------------- //
// child-is traversal with a learned child order, and its sample recorder     //
// ------------------------------------------------------------------------- //
//
// The plain order visits the child with the smaller entry distance first
// (kernels.cu:818-827).  LEARNED asks the network instead at every node
// where both children are hit and not culled; every such child is still
// visited, so the closest hit is the same (up to which of two triangles at
// exactly the same t is found first).  SAMPLE keeps the plain order and
// records each such decision for training.  Lanes converge once per step so
// that the warp evaluates the network for all deciding lanes at once on the
// tensor cores.

struct LearnArgs {
    TraceArgs t;
    const MlpWeights *w;
    Sample *samples;
    uint32_t *sample_count;
    uint32_t sample_cap;
    const HitRec *hint;   // HINT: each ray's known closest hit
};

__device__ __forceinline__ float clampf4(float v) { return fminf(fmaxf(v, -4.0f), 4.0f); }

// HINT replaces the network by the ideal decision: the child whose Morton
// range holds the ray's known closest hit goes first (the plain order where
// the ray misses).  No predictor can do better than this order, so it bounds
// what a learned order may gain.
template <bool SAMPLE, bool LEARNED, bool STATS, int STACK, bool HINT = false>
__global__ void __launch_bounds__(kTraceThreads) k_trace_learn(LearnArgs L)
{
    const TraceArgs &A = L.t;
    __shared__ MlpWeights sw;
    __shared__ __align__(16) __nv_bfloat16 xs[kTraceThreads / 32][32][kMlpIn];
    if (LEARNED) {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(L.w);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sw);
        for (int i = threadIdx.x; i < (int)(sizeof(MlpWeights) / 4); i += blockDim.x) dst[i] = src[i];
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t nrays = A.d_nrays ? *A.d_nrays : A.nrays;
    const RootRec root = *A.root;
    const uint32_t n_inner = A.n_tris - 1u;

    bool active = false, exhausted = false;
    uint32_t r = 0, cur = 0, depth = 0, steps = 0, inner_visits = 0, tri_tests = 0;
    int sp = -1;
    uint32_t stack[STACK];
    Ray R;
    Best best;
    bool overflow = false, capped = false, bad = false;
    uint32_t hint_ref = 0xffffffffu;   // HINT: Morton position of the known hit
    bool parked = false;        // LEARNED: waiting for the warp's next network pass
    uint32_t pq_l = 0, pq_r = 0;   // child links of the parked decision
    bool pq_plain = false;         // the plain rule's choice there: left first
    uint32_t px[kMlpIn / 2];    // its features, packed bf16 pairs

    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && __popc(idle) >= kFetchIdle) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(A.queue, (uint32_t)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base >= nrays) {
                exhausted = true;
            } else if (!active) {
                r = base + __popc(idle & lt_mask);
                if (r < nrays) {
                    float o[3], d[3];
                    for (int k = 0; k < 3; ++k) {
                        o[k] = A.orig[3 * (size_t)r + k];
                        d[k] = A.dir[3 * (size_t)r + k];
                    }
                    make_ray(R, o, d, A.maxt[r]);
                    if (HINT) {
                        const HitRec h = L.hint[r];
                        hint_ref = h.t != FLT_MAX ? h.ref : 0xffffffffu;
                    }
                    best.t = FLT_MAX;
                    best.beta = best.gamma = 0.f;
                    best.ref = 0;
                    sp = -1;
                    steps = inner_visits = tri_tests = depth = 0;
                    cur = root.link;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }

        bool done = false, at_inner = false, need = false, hl = false, hr = false;
        NodeRec nd;
        float tnl = FLT_MAX, tfl = FLT_MAX, tnr = FLT_MAX, tfr = FLT_MAX;
        const bool stepping = active && !parked;   // a parked lane waits this step out
        if (stepping) {
            if (++steps > kMaxSteps) {
                capped = true;
                done = true;
            } else if (!is_leaf(cur)) {
                if (cur >= n_inner) {
                    bad = true;
                    done = true;
                } else {
                    at_inner = true;
                    ++inner_visits;
                    nd = load_node(A.nodes, cur);
                    hl = slab_test(RTA_LEFT_BOX(nd), R, tnl, tfl);
                    hr = slab_test(RTA_RIGHT_BOX(nd), R, tnr, tfr);
                    if (tnl >= best.t || tnl > R.tmax) hl = false;
                    if (tnr >= best.t || tnr > R.tmax) hr = false;
                    // only overlapping entry-exit intervals make the order
                    // matter: when the nearer child's interval ends before
                    // the farther one begins, nearer-first is never worse
                    need = hl && hr && (tnl <= tnr ? tnr < tfl : tnl < tfr);
                }
            }
        }
        bool left_first = tnl <= tnr;
        if (HINT && need && hint_ref != 0xffffffffu) {
            const uint32_t lfirst = is_leaf(nd.q3.x) ? leaf_first(nd.q3.x) : nd.q3.x - nd.q3.z + 1u;
            const uint32_t rfirst = is_leaf(nd.q3.y) ? leaf_first(nd.q3.y) : nd.q3.y;
            if (hint_ref - lfirst < nd.q3.z) left_first = true;
            else if (hint_ref - rfirst < nd.q3.w) left_first = false;
        }
        if (SAMPLE || LEARNED) {
            if (need) {
                float x[kMlpIn];
                const float base = fminf(tnl, tnr), span = fmaxf(tfl, tfr) - base;
                const float inv = span > 0.0f ? 1.0f / span : 0.0f;
                x[0] = clampf4(R.d[0]);
                x[1] = clampf4(R.d[1]);
                x[2] = clampf4(R.d[2]);
                x[3] = clampf4((tnl - base) * inv);
                x[4] = clampf4((tfl - base) * inv);
                x[5] = clampf4((tnr - base) * inv);
                x[6] = clampf4((tfr - base) * inv);
                x[7] = (float)depth * (1.0f / 32.0f);
                x[8] = log2f((float)nd.q3.z) * (1.0f / 25.0f);
                x[9] = log2f((float)nd.q3.w) * (1.0f / 25.0f);
                x[10] = best.t != FLT_MAX ? 1.0f : 0.0f;
                x[11] = best.t != FLT_MAX ? clampf4((best.t - base) * inv) * 0.25f : 1.0f;
                x[12] = (is_leaf(nd.q3.x) ? 1.0f : 0.0f) - (is_leaf(nd.q3.y) ? 1.0f : 0.0f);
                x[13] = tnl <= tnr ? 1.0f : -1.0f;
                x[14] = x[15] = 0.0f;
#pragma unroll
                for (int k = 0; k < kMlpIn / 2; ++k) px[k] = pack_bf16(x[k * 2], x[k * 2 + 1]);
            }
            if (SAMPLE) {
                const uint32_t m = __ballot_sync(0xffffffffu, need);
                if (m) {
                    const int leader = __ffs(m) - 1;
                    uint32_t base = 0;
                    if ((int)lane == leader) base = atomicAdd(L.sample_count, (uint32_t)__popc(m));
                    base = __shfl_sync(0xffffffffu, base, leader);
                    const uint32_t idx = base + __popc(m & lt_mask);
                    if (need && idx < L.sample_cap) {
                        Sample smp;
#pragma unroll
                        for (int k = 0; k < kMlpIn / 2; ++k)
                            *reinterpret_cast<uint32_t *>(&smp.x[2 * k]) = px[k];
                        smp.ray = r;
                        smp.lsize = nd.q3.z;
                        smp.rsize = nd.q3.w;
                        smp.lfirst = is_leaf(nd.q3.x) ? leaf_first(nd.q3.x) : nd.q3.x - nd.q3.z + 1u;
                        smp.rfirst = is_leaf(nd.q3.y) ? leaf_first(nd.q3.y) : nd.q3.y;
                        smp.label = 0.f;
                        smp.weight = 0.f;
                        smp.pad = 0;
                        L.samples[idx] = smp;
                    }
                }
            }
            if (LEARNED) {
                // a deciding lane parks with its features and both child links
                // until enough lanes of the warp (or all its active ones) wait,
                // then one tensor-core pass decides for all of them
                if (need) {
                    parked = true;
                    pq_l = nd.q3.x;
                    pq_r = nd.q3.y;
                    pq_plain = tnl <= tnr;
                }
                const uint32_t pm = __ballot_sync(0xffffffffu, parked);
                if (pm && (__popc(pm) >= kParkMin || pm == __ballot_sync(0xffffffffu, active))) {
#pragma unroll
                    for (int k = 0; k < kMlpIn / 2; ++k)
                        *reinterpret_cast<uint32_t *>(&xs[warp][lane][2 * k]) = parked ? px[k] : 0u;
                    __syncwarp();
                    MlpForward F;
                    mlp_forward(sw, xs[warp], F);
                    const float logit = mlp_own_logit(F);
                    __syncwarp();
                    if (parked) {
                        parked = false;
                        if (sp + 1 >= STACK) {
                            overflow = true;
                            done = true;
                        } else {
                            // a confident network decides; below the margin
                            // the plain nearer-first rule does
                            const bool lf = fabsf(logit) > sw.margin ? logit > 0.0f : pq_plain;
                            const uint32_t far = lf ? pq_r : pq_l;
                            const uint32_t d1 = depth + 1u < 63u ? depth + 1u : 63u;
                            stack[++sp] = is_leaf(far) ? far : (far | (d1 << kCountShift));
                            cur = lf ? pq_l : pq_r;
                            depth = d1;
                        }
                    }
                }
            }
        }
        if (stepping && !done && !(LEARNED && need)) {
            if (at_inner) {
                if (hl && hr) {
                    if (sp + 1 >= STACK) {
                        overflow = true;
                        done = true;
                    } else {
                        const uint32_t far = left_first ? nd.q3.y : nd.q3.x;
                        const uint32_t d1 = depth + 1u < 63u ? depth + 1u : 63u;
                        stack[++sp] = is_leaf(far) ? far : (far | (d1 << kCountShift));
                        cur = left_first ? nd.q3.x : nd.q3.y;
                        depth = d1;
                    }
                } else if (hl) {
                    cur = nd.q3.x;
                    depth = depth + 1u < 63u ? depth + 1u : 63u;
                } else if (hr) {
                    cur = nd.q3.y;
                    depth = depth + 1u < 63u ? depth + 1u : 63u;
                } else if (sp < 0) {
                    done = true;
                } else {
                    const uint32_t e = stack[sp--];
                    cur = is_leaf(e) ? e : (e & kFirstMask);
                    if (!is_leaf(e)) depth = (e >> kCountShift) & kCountMask;
                }
            } else {
                if (visit_leaf<false>(A.tris, A.n_tris, cur, R.o, R.d, R.tmax, best, tri_tests, bad))
                    done = true;
                else if (sp < 0)
                    done = true;
                else {
                    const uint32_t e = stack[sp--];
                    cur = is_leaf(e) ? e : (e & kFirstMask);
                    if (!is_leaf(e)) depth = (e >> kCountShift) & kCountMask;
                }
            }
        }
        if (done) {
            if (best.t != FLT_MAX) {
                reinterpret_cast<float4 *>(A.hits)[r] =
                    make_float4(best.t, best.beta, best.gamma, __uint_as_float(best.ref));
            } else {
                A.hits[r].t = FLT_MAX;
            }
            if (STATS) {
                A.stats[2 * (size_t)r + 0] = inner_visits;
                A.stats[2 * (size_t)r + 1] = tri_tests;
            }
            active = false;
        }
    }
    if (overflow) atomicOr(A.status, RTA_DEV_STACK_OVERFLOW);
    if (capped) atomicOr(A.status, RTA_DEV_ITER_LIMIT);
    if (bad) atomicOr(A.status, RTA_DEV_BAD_LINK);
}

template <bool SAMPLE, bool LEARNED, bool STATS, int STACK, bool HINT = false>
static int launch_learn(const LearnArgs &a, cudaStream_t s)
{
    static int blocks = 0;
    if (!blocks) {
        int per_sm = 0, dev = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_learn<SAMPLE, LEARNED, STATS, STACK, HINT>,
                                                      kTraceThreads, 0);
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    }
    k_trace_learn<SAMPLE, LEARNED, STATS, STACK, HINT><<<blocks, kTraceThreads, 0, s>>>(a);
    return check_launch("k_trace_learn");
}

template <int STACK>
static int dispatch_learn(const LearnArgs &a, bool sample, bool learned, bool stats, cudaStream_t s)
{
    if (a.hint)
        return stats ? launch_learn<false, false, true, STACK, true>(a, s)
                     : launch_learn<false, false, false, STACK, true>(a, s);
    if (sample) return launch_learn<true, false, false, STACK>(a, s);
    if (learned) return stats ? launch_learn<false, true, true, STACK>(a, s) : launch_learn<false, true, false, STACK>(a, s);
    return stats ? launch_learn<false, false, true, STACK>(a, s) : launch_learn<false, false, false, STACK>(a, s);
}

int trace_learn_impl(const rta_lbvh *bvh, const MlpWeights *w, const float *orig, const float *dir,
                     const float *maxt, uint32_t nrays, const uint32_t *d_nrays, void *hits,
                     uint32_t *stats, Sample *samples, uint32_t *sample_count, uint32_t sample_cap,
                     uint32_t *queue, bool learned, cudaStream_t s, const void *hint)
{
    LearnArgs a;
    a.t.nodes = (const NodeRec *)bvh->nodes;
    a.t.root = (const RootRec *)bvh->root;
    a.t.tris = (const TriRec *)bvh->tris;
    a.t.orig = orig;
    a.t.dir = dir;
    a.t.maxt = maxt;
    a.t.nrays = nrays;
    a.t.d_nrays = d_nrays;
    a.t.hits = (HitRec *)hits;
    a.t.stats = stats;
    a.t.queue = queue;
    a.t.status = bvh->status;
    a.t.n_tris = bvh->n;
    a.w = w;
    a.samples = samples;
    a.sample_count = sample_count;
    a.sample_cap = sample_cap;
    a.hint = (const HitRec *)hint;
    RTA_CUDA_TRY(cudaMemsetAsync(queue, 0, 4, s));
    const bool sample = samples != nullptr;
    if (bvh->morton_bits == 63) return dispatch_learn<80>(a, sample, learned, stats != nullptr, s);
    return dispatch_learn<40>(a, sample, learned, stats != nullptr, s);
}

template <bool DIS, bool SHADOW, bool AILA, bool STATS, int STACK>
static int launch_trace(const TraceArgs &a, cudaStream_t s)
{
    static int blocks = 0;
    if (!blocks) {
        int per_sm = 0, dev = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<DIS, SHADOW, AILA, STATS, STACK>, kTraceThreads, 0);
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    }
    k_trace<DIS, SHADOW, AILA, STATS, STACK><<<blocks, kTraceThreads, 0, s>>>(a);
    return check_launch("k_trace");
}

// The frame's primary pass with each bounce ray traced right after its
// primary ray (child-is closest hit).  b_* are per-primary-ray slots.
template <int STACK>
static int launch_fused(const TraceArgs &a, cudaStream_t s)
{
    static int blocks = 0;
    if (!blocks) {
        int per_sm = 0, dev = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<false, false, false, false, STACK, true>,
                                                      kTraceThreads, 0);
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    }
    k_trace<false, false, false, false, STACK, true><<<blocks, kTraceThreads, 0, s>>>(a);
    return check_launch("k_trace fused frame");
}

int trace_frame_fused(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt, uint32_t nrays,
                      void *hits, uint32_t seed, float eps, float *b_orig, float *b_dir, void *b_hits,
                      uint32_t *b_flag, uint32_t *b_tile, uint32_t *queue, cudaStream_t s)
{
    TraceArgs a;
    a.nodes = (const NodeRec *)bvh->nodes;
    a.root = (const RootRec *)bvh->root;
    a.tris = (const TriRec *)bvh->tris;
    a.orig = orig;
    a.dir = dir;
    a.maxt = maxt;
    a.nrays = nrays;
    a.d_nrays = nullptr;
    a.hits = (HitRec *)hits;
    a.stats = nullptr;
    a.queue = queue;
    a.status = bvh->status;
    a.n_tris = bvh->n;
    a.seed = seed;
    a.eps = eps;
    a.b_orig = b_orig;
    a.b_dir = b_dir;
    a.b_hits = (HitRec *)b_hits;
    a.b_flag = b_flag;
    a.b_tile = b_tile;   // the caller zeroes *queue and b_tile
    return bvh->morton_bits == 63 ? launch_fused<80>(a, s) : launch_fused<40>(a, s);
}

template <int STACK>
static int dispatch(const TraceArgs &a, uint32_t mode, cudaStream_t s)
{
    const bool dis = mode & RTA_TRACE_DIS, sh = mode & RTA_TRACE_SHADOW, ai = mode & RTA_TRACE_AILA,
               st = mode & RTA_TRACE_STATS;
#define RTA_CASE(D, S, A, T) \
    if (dis == D && sh == S && ai == A && st == T) return launch_trace<D, S, A, T, STACK>(a, s);
    RTA_CASE(false, false, false, false) RTA_CASE(false, false, false, true)
    RTA_CASE(false, true, false, false) RTA_CASE(false, true, false, true)
    RTA_CASE(false, false, true, false) RTA_CASE(false, false, true, true)
    RTA_CASE(false, true, true, false) RTA_CASE(false, true, true, true)
    RTA_CASE(true, false, false, false) RTA_CASE(true, false, false, true)
    RTA_CASE(true, true, false, false) RTA_CASE(true, true, false, true)
    RTA_CASE(true, false, true, false) RTA_CASE(true, false, true, true)
    RTA_CASE(true, true, true, false) RTA_CASE(true, true, true, true)
#undef RTA_CASE
    return RTA_ERR_INVALID;
}

// the tree depth after the equal-code collapse is at most the number of code
// bits + 1, which bounds the stack (one push per level)
int trace_impl(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt,
               uint32_t nrays, const uint32_t *d_nrays, void *hits, uint32_t mode, uint32_t *stats,
               uint32_t *queue, cudaStream_t s)
{
    TraceArgs a;
    a.nodes = (const NodeRec *)bvh->nodes;
    a.root = (const RootRec *)bvh->root;
    a.tris = (const TriRec *)bvh->tris;
    a.orig = orig;
    a.dir = dir;
    a.maxt = maxt;
    a.nrays = nrays;
    a.d_nrays = d_nrays;
    a.hits = (HitRec *)hits;
    a.stats = stats;
    a.queue = queue;
    a.status = bvh->status;
    a.n_tris = bvh->n;
    RTA_CUDA_TRY(cudaMemsetAsync(queue, 0, 4, s));
    if (bvh->morton_bits == 63) return dispatch<80>(a, mode, s);
    return dispatch<40>(a, mode, s);
}

} // namespace rta

using namespace rta;

extern "C" int rta_trace(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt,
                         uint32_t nrays, const uint32_t *d_nrays, void *hits, uint32_t mode,
                         uint32_t *stats, rta_stream_t stream)
{
    if (!bvh || !orig || !dir || !maxt || !hits || (!d_nrays && nrays == 0)) return RTA_ERR_INVALID;
    if ((mode & RTA_TRACE_STATS) && !stats) return RTA_ERR_INVALID;
    // the queue word lives after the status word in the context's status block
    uint32_t *queue = bvh->status + 4;
    return trace_impl(bvh, orig, dir, maxt, nrays, d_nrays, hits, mode, stats, queue,
                      (cudaStream_t)stream);
}
