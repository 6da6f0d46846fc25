/*
 * oracle.c -- CPU restatement of rta's LBVH build and binary-BVH traversal.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  It is called by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
 * product.  Build with -ffp-contract=off so that every floating-point
 * expression is evaluated exactly as the reference source writes it.
 *
 * References are to files of kiselgra/rta (path:line).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TRI ORC_TRI_FLOATS
#define NODE ORC_NODE_FLOATS

/* The reference's MIN/MAX macros (lbvh-kernels.cu:142-143, :259-260). */
static inline float ref_min(float a, float b) { return (a < b) ? a : b; }
static inline float ref_max(float a, float b) { return (a > b) ? a : b; }

static inline uint32_t f_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bits_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }
static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

/* float -> unsigned conversion with the GPU's cvt.rzi.u32.f32 semantics:
 * truncation toward zero, NaN and negatives give 0, overflow saturates.  The
 * reference writes `uint x = center.x * d.x;` (lbvh-kernels.cu:177) and runs
 * it on the GPU, so this is the behaviour its codes have.                  */
static inline uint32_t f2u_rz_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)v;
}

/* ------------------------------------------------------------------------ */
/* Morton codes                                                              */
/* ------------------------------------------------------------------------ */

/* spread the low 10 bits of v so that bit k lands on bit 3k */
static inline uint32_t spread3_10(uint32_t v)
{
    uint32_t r = 0;
    for (int k = 0; k < 10; ++k) r |= ((v >> k) & 1u) << (3 * k);
    return r;
}

/* spread the low 21 bits of v so that bit k lands on bit 3k */
static inline uint64_t spread3_21(uint64_t v)
{
    uint64_t r = 0;
    for (int k = 0; k < 21; ++k) r |= ((v >> k) & 1ull) << (3 * k);
    return r;
}

void orc_centroid(const float *t, float out[3])
{
    /* (tri.a+tri.b+tri.c)/3.0f, lbvh-kernels.cu:60-63 */
    for (int k = 0; k < 3; ++k) {
        float s = t[k] + t[3 + k];
        s = s + t[6 + k];
        out[k] = s / 3.0f;
    }
}

uint64_t orc_morton(const float c[3], const float mn[3], const float d[3], int bits,
                    uint32_t *flags)
{
    /* morton_codes2 (lbvh-kernels.cu:169-183): center - c, times d, (uint),
     * masked interleave; x -> bit 0, y -> bit 1, z -> bit 2 (:99-129).  For
     * 63-bit codes the same recipe runs with a 2^21 grid.                   */
    const uint32_t grid = (bits == 63) ? (1u << 21) : (1u << 10);
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        float rel = c[k] - mn[k];
        float s = rel * d[k];
        q[k] = f2u_rz_sat(s);
        if (flags && q[k] >= grid) *flags |= ORC_FLAG_WRAP;
        q[k] &= grid - 1u;
    }
    if (bits == 63)
        return spread3_21(q[0]) | (spread3_21(q[1]) << 1) | (spread3_21(q[2]) << 2);
    return (uint64_t)(spread3_10(q[0]) | (spread3_10(q[1]) << 1) | (spread3_10(q[2]) << 2));
}

/* ------------------------------------------------------------------------ */
/* stable LSD radix sort of (key, id) pairs (stands for thrust::sort_by_key, */
/* lbvh-kernels.cu:537-555, which is a stable radix sort for integer keys)  */
/* ------------------------------------------------------------------------ */

static void radix_sort_pairs(uint64_t *key, uint32_t *val, uint32_t n, int bits)
{
    uint64_t *k2 = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
    uint32_t *v2 = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        size_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        int sh = 8 * p;
        for (uint32_t i = 0; i < n; ++i) cnt[((key[i] >> sh) & 0xff) + 1]++;
        for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
        for (uint32_t i = 0; i < n; ++i) {
            size_t dst = cnt[(key[i] >> sh) & 0xff]++;
            k2[dst] = key[i];
            v2[dst] = val[i];
        }
        memcpy(key, k2, (size_t)n * sizeof(uint64_t));
        memcpy(val, v2, (size_t)n * sizeof(uint32_t));
    }
    free(k2);
    free(v2);
}

/* ------------------------------------------------------------------------ */
/* Karras radix tree (lbvh-kernels.cu:84-96, 186-256)                        */
/* ------------------------------------------------------------------------ */

/* common prefix length with the index tie-break (`__cpl`, :84-92) */
static inline int cpl(const uint64_t *codes, int n, int m1, int m2, int wide)
{
    if (m2 < 0 || m2 >= n) return -1;
    if (codes[m1] == codes[m2]) return (wide ? 64 : 32) + clz32((uint32_t)(m1 ^ m2));
    if (wide) return clz64(codes[m1] ^ codes[m2]);
    return clz32((uint32_t)(codes[m1] ^ codes[m2]));
}

static inline int ref_sign(int v) { return (v >= 0) ? 1 : -1; }
static inline int div2ceil(int v) { return v / 2 + v % 2; }

/* node field helpers on the 2F4 layout */
static inline void node_set_inner(float *nd, uint32_t l, uint32_t r)
{
    nd[0] = bits_f((l << 1) | 1u);
    nd[1] = bits_f(r);
}
static inline void node_set_leaf(float *nd, uint32_t tris, uint32_t elems)
{
    nd[0] = bits_f(elems << 1);
    nd[1] = bits_f(tris);
}
static inline int node_inner(const float *nd) { return (f_bits(nd[0]) & 1u) == 1u; }
static inline uint32_t node_left(const float *nd) { return f_bits(nd[0]) >> 1; }
static inline uint32_t node_right(const float *nd) { return f_bits(nd[1]); }

static void karras_node(const uint64_t *codes, int n, int i, int wide, uint32_t *left,
                        uint32_t *right)
{
    int d = ref_sign(cpl(codes, n, i, i + 1, wide) - cpl(codes, n, i, i - 1, wide));
    int cpl_min = cpl(codes, n, i, i - d, wide);
    int l_max = 2;
    while (cpl(codes, n, i, i + l_max * d, wide) > cpl_min) l_max = l_max * 2;
    int l = 0;
    for (int t = l_max / 2; t >= 1; t = t / 2)
        if (cpl(codes, n, i, i + (l + t) * d, wide) > cpl_min) l = l + t;
    int j = i + l * d;
    int from = i, to = j;
    if (j < i) { from = j; to = i; }
    int cpl_node = cpl(codes, n, from, to, wide);
    int s = 0;
    for (int t = div2ceil(l); t >= 1; t = div2ceil(t)) {
        if (cpl(codes, n, from, from + (s + t), wide) > cpl_node) s = s + t;
        if (t <= 1) break;
    }
    int mid = from + s;
    int lft = mid, rgt = mid + 1;
    if (from == mid) lft += n - 1;
    if (to == mid + 1) rgt += n - 1;
    *left = (uint32_t)lft;
    *right = (uint32_t)rgt;
}

/* ------------------------------------------------------------------------ */
/* LBVH build                                                                */
/* ------------------------------------------------------------------------ */

static void tri_box(const float *t, float mn[3], float mx[3])
{
    /* aabbOfTri (lbvh-kernels.cu:141-153): MIN(MIN(a,b),c), MAX(MAX(a,b),c) */
    for (int k = 0; k < 3; ++k) {
        mn[k] = ref_min(ref_min(t[k], t[3 + k]), t[6 + k]);
        mx[k] = ref_max(ref_max(t[k], t[3 + k]), t[6 + k]);
    }
}

int orc_lbvh_build(const float *tris, uint32_t n, int bits, uint64_t *codes, uint32_t *ids,
                   float *nodes, float *scene, float *scale, uint32_t *flags)
{
    if (n == 0 || (bits != 30 && bits != 63) || n > 0x3fffffffu) return -1;
    uint32_t fl = 0;
    const int wide = (bits == 63);
    const float grid = wide ? 2097152.0f : 1024.0f;

    /* K1 + K2: triangle boxes and the scene box (init +-1e11, :519-520) */
    float smin[3] = {100000000000.0f, 100000000000.0f, 100000000000.0f};
    float smax[3] = {-100000000000.0f, -100000000000.0f, -100000000000.0f};
    for (uint32_t i = 0; i < n; ++i) {
        float mn[3], mx[3];
        tri_box(tris + (size_t)i * TRI, mn, mx);
        for (int k = 0; k < 3; ++k) {
            smin[k] = ref_min(smin[k], mn[k]);
            smax[k] = ref_max(smax[k], mx[k]);
        }
    }
    float d[3];
    for (int k = 0; k < 3; ++k) {
        /* host side, lbvh-kernels.cu:414-417 */
        d[k] = grid / (smax[k] - smin[k]);
        if (!isfinite(d[k])) fl |= ORC_FLAG_NONFINITE;
        scene[k] = smin[k];
        scene[3 + k] = smax[k];
        scale[k] = d[k];
    }

    /* K3: codes, ids = identity */
    for (uint32_t i = 0; i < n; ++i) {
        float c[3];
        orc_centroid(tris + (size_t)i * TRI, c);
        codes[i] = orc_morton(c, smin, d, bits, &fl);
        ids[i] = i;
    }
    /* K4: stable sort by code */
    radix_sort_pairs(codes, ids, n, wide ? 64 : 32);

    /* K5: tree links and parents */
    const uint32_t nn = 2 * n - 1;
    uint32_t *parent = (uint32_t *)malloc((size_t)nn * sizeof(uint32_t));
    uint32_t *counter = (uint32_t *)calloc(n, sizeof(uint32_t));
    memset(nodes, 0, (size_t)nn * NODE * sizeof(float));
    parent[0] = 0;
    for (uint32_t i = 0; i < nn; ++i) {
        float *nd = nodes + (size_t)i * NODE;
        if (i >= n - 1) {
            node_set_leaf(nd, i - (n - 1), 1);
            continue;
        }
        uint32_t l, r;
        karras_node(codes, (int)n, (int)i, wide, &l, &r);
        node_set_inner(nd, l, r);
        parent[l] = i;
        parent[r] = i;
    }

    /* K6: bottom-up refit with equal-code leaf collapse.  The reference uses the
     * child's Morton code as the first-arrival token (:285-291); here arrivals
     * are counted, which gives the same tree whenever no code is 0.         */
#define CODE_OF(idx) (((idx) >= n - 1) ? codes[(idx) - (n - 1)] : codes[(idx)])
    for (uint32_t j = 0; j < n; ++j) {
        uint32_t cur = j + (n - 1);
        float bmn[3], bmx[3];
        tri_box(tris + (size_t)ids[j] * TRI, bmn, bmx);
        float *nd = nodes + (size_t)cur * NODE;
        for (int k = 0; k < 3; ++k) { nd[2 + k] = bmn[k]; nd[5 + k] = bmx[k]; }
        while (cur != 0) {
            uint32_t last = cur;
            uint64_t code = CODE_OF(cur);
            cur = parent[cur];
            if (counter[cur]++ == 0) break; /* first arrival stops */
            float *p = nodes + (size_t)cur * NODE;
            uint32_t sib = (node_left(p) == last) ? node_right(p) : node_left(p);
            uint64_t old = CODE_OF(sib);
            if (code == 0 || old == 0) fl |= ORC_FLAG_CODE0_RACE;
            const float *s = nodes + (size_t)sib * NODE;
            for (int k = 0; k < 3; ++k) {
                bmn[k] = ref_min(bmn[k], s[2 + k]);
                bmx[k] = ref_max(bmx[k], s[5 + k]);
            }
            for (int k = 0; k < 3; ++k) { p[2 + k] = bmn[k]; p[5 + k] = bmx[k]; }
            if (code == old) {
                const float *rn = nodes + (size_t)node_right(p) * NODE;
                const float *ln = nodes + (size_t)node_left(p) * NODE;
                if (!node_inner(rn) && !node_inner(ln)) {
                    uint32_t rt = f_bits(rn[1]), lt = f_bits(ln[1]);
                    uint32_t tr = (rt < lt) ? rt : lt;
                    uint32_t len = (f_bits(rn[0]) >> 1) + (f_bits(ln[0]) >> 1);
                    node_set_leaf(p, tr, len);
                }
            }
        }
    }
#undef CODE_OF
    free(parent);
    free(counter);
    if (!wide && n > 1 && codes[0] == 0) fl |= ORC_FLAG_CODE0_RACE;
    if (flags) *flags = fl;
    return 0;
}

void orc_permute(const float *tris, const uint32_t *ids, uint32_t n, float *out)
{
    for (uint32_t k = 0; k < n; ++k)
        memcpy(out + (size_t)k * TRI, tris + (size_t)ids[k] * TRI, TRI * sizeof(float));
}

/* ------------------------------------------------------------------------ */
/* intersection tests (librta/intersect.h)                                   */
/* ------------------------------------------------------------------------ */

int orc_intersect_tri(const float *tri, const float o[3], const float dir[3], float *tout,
                      float *bout, float *gout)
{
    /* intersect_tri_opt, intersect.h:8-53, expression for expression */
    float a_x = tri[0], a_y = tri[1], a_z = tri[2];
    float a = a_x - tri[3];
    float b = a_y - tri[4];
    float c = a_z - tri[5];
    float d = a_x - tri[6];
    float e = a_y - tri[7];
    float f = a_z - tri[8];
    float g = dir[0], h = dir[1], i = dir[2];
    float j = a_x - o[0];
    float k = a_y - o[1];
    float l = a_z - o[2];
    float common1 = e * i - h * f;
    float common2 = g * f - d * i;
    float common3 = d * h - e * g;
    float M = a * common1 + b * common2 + c * common3;
    float beta = j * common1 + k * common2 + l * common3;
    common1 = a * k - j * b;
    common2 = j * c - a * l;
    common3 = b * l - k * c;
    float gamma = i * common1 + h * common2 + g * common3;
    float tt = -(f * common1 + e * common2 + d * common3);
    beta /= M;
    gamma /= M;
    tt /= M;
    if (tt > 0)
        if (beta > 0 && gamma > 0 && beta + gamma <= 1) {
            *tout = tt;
            *bout = beta;
            *gout = gamma;
            return 1;
        }
    return 0;
}

int orc_intersect_aabb(const float bmin[3], const float bmax[3], const float o[3],
                       const float d[3], float *dist)
{
    /* intersect_aabb, intersect.h:56-150 */
    float t_near = -FLT_MAX, t_far = FLT_MAX;
    for (int k = 0; k < 3; ++k) {
        const float dk = d[k], ek = o[k];
        if (dk == 0) {
            if (ek < bmin[k] || ek > bmax[k]) return 0;
        } else {
            float t1 = (bmin[k] - ek) / dk;
            float t2 = (bmax[k] - ek) / dk;
            if (t1 > t2) { float tmp = t1; t1 = t2; t2 = tmp; }
            if (t1 > t_near) t_near = t1;
            if (t2 < t_far) t_far = t2;
            if (t_near > t_far) return 0;
            if (t_far < 0) return 0;
        }
    }
    *dist = t_near;
    return 1;
}

/* intersect_aabb_aila (intersect.h:165-176) with the reciprocal direction of
 * the ailabox kernels (kernels.cu:966-970) */
static int aabb_aila(const float mi[3], const float ma[3], const float o[3], const float id[3],
                     float t, float *ret)
{
    float t1[3], t2[3];
    for (int k = 0; k < 3; ++k) {
        float oid = o[k] * id[k];
        t1[k] = (mi[k] * id[k]) - oid;
        t2[k] = (ma[k] * id[k]) - oid;
    }
    float near = fmaxf(fmaxf(fminf(t1[0], t2[0]), fminf(t1[1], t2[1])), fminf(t1[2], t2[2]));
    float far = fminf(fminf(fmaxf(t1[0], t2[0]), fmaxf(t1[1], t2[1])), fmaxf(t1[2], t2[2]));
    *ret = near;
    return near <= far && far >= 0.f && near < t;
}

/* ------------------------------------------------------------------------ */
/* traversal of the reference 2F4 layout (bbvh-cuda/kernels.cu)              */
/* ------------------------------------------------------------------------ */

static inline void node_box(const float *nodes, uint32_t idx, float mn[3], float mx[3])
{
    const float *nd = nodes + (size_t)idx * NODE;
    mn[0] = nd[2]; mn[1] = nd[3]; mn[2] = nd[4];
    mx[0] = nd[5]; mx[1] = nd[6]; mx[2] = nd[7];
}

static int trace_one(const float *nodes, const float *tris, const float o[3], const float dir[3],
                     float t_max, int mode, int stack_limit, orc_hit *hit, uint32_t *st)
{
    const int shadow = (mode & ORC_SHADOW) != 0;
    const int dis = (mode & ORC_DIS) != 0;
    const int aila = (mode & ORC_AILA) != 0;
    uint32_t stack[256];
    int sp = -1;
    uint32_t inner_visits = 0, tri_tests = 0;
    orc_hit closest = *hit;
    closest.t = FLT_MAX;
    float idir[3] = {0, 0, 0};
    if (aila) {
        const float ooeps = 8.27180612553027674871e-25f; /* 2^-80 */
        for (int k = 0; k < 3; ++k)
            idir[k] = 1.0f / (fabsf(dir[k]) > ooeps ? dir[k] : copysignf(ooeps, dir[k]));
    }
    int overflow = 0;
    uint32_t cur = 0;
    float dist_l = FLT_MAX, dist_r = FLT_MAX, dist = FLT_MAX;
    for (;;) {
        const float *nd = nodes + (size_t)cur * NODE;
        if (node_inner(nd)) {
            inner_visits++;
            if (dis) {
                /* kernels.cu:506-529 */
                float mn[3], mx[3];
                node_box(nodes, cur, mn, mx);
                int h = aila ? aabb_aila(mn, mx, o, idir, closest.t, &dist)
                             : orc_intersect_aabb(mn, mx, o, dir, &dist);
                if (dist >= closest.t || dist > t_max) h = 0;
                if (h) {
                    if (sp + 1 >= stack_limit) { overflow = 1; break; }
                    stack[++sp] = node_right(nd);
                    cur = node_left(nd);
                } else if (sp >= 0)
                    cur = stack[sp--];
                else
                    break;
            } else {
                /* kernels.cu:797-835 */
                uint32_t L = node_left(nd), R = node_right(nd);
                float mn[3], mx[3];
                node_box(nodes, L, mn, mx);
                int hl = aila ? aabb_aila(mn, mx, o, idir, closest.t, &dist_l)
                              : orc_intersect_aabb(mn, mx, o, dir, &dist_l);
                node_box(nodes, R, mn, mx);
                int hr = aila ? aabb_aila(mn, mx, o, idir, closest.t, &dist_r)
                              : orc_intersect_aabb(mn, mx, o, dir, &dist_r);
                if (dist_l >= closest.t || dist_l > t_max) hl = 0;
                if (dist_r >= closest.t || dist_r > t_max) hr = 0;
                if (hl) {
                    if (hr) {
                        if (sp + 1 >= stack_limit) { overflow = 1; break; }
                        if (dist_l <= dist_r) { stack[++sp] = R; cur = L; }
                        else { stack[++sp] = L; cur = R; }
                    } else
                        cur = L;
                } else if (hr)
                    cur = R;
                else if (sp >= 0)
                    cur = stack[sp--];
                else
                    break;
            }
        } else {
            uint32_t elems = f_bits(nd[0]) >> 1;
            uint32_t offset = f_bits(nd[1]);
            for (uint32_t i = 0; i < elems; ++i) {
                float t, b, g;
                tri_tests++;
                if (orc_intersect_tri(tris + (size_t)(offset + i) * TRI, o, dir, &t, &b, &g)) {
                    if (t < closest.t && t <= t_max) {
                        closest.t = t;
                        closest.beta = b;
                        closest.gamma = g;
                        closest.ref = offset + i;
                        if (shadow) break;
                    }
                }
            }
            if (shadow && closest.t != FLT_MAX) break;
            if (sp >= 0)
                cur = stack[sp--];
            else
                break;
        }
    }
    *hit = closest;
    if (st) { st[0] = inner_visits; st[1] = tri_tests; }
    return overflow;
}

int orc_trace(const float *nodes, const float *tris, const float *orig, const float *dir,
              const float *maxt, uint32_t nrays, int mode, int stack_limit, orc_hit *hits,
              uint32_t *stats, int threads)
{
    if (stack_limit <= 0 || stack_limit > 256) stack_limit = 256;
    int bad = 0;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) reduction(| : bad)
#endif
    for (long long i = 0; i < (long long)nrays; ++i) {
        bad |= trace_one(nodes, tris, orig + 3 * i, dir + 3 * i, maxt[i], mode, stack_limit,
                         hits + i, stats ? stats + 2 * i : NULL);
    }
    (void)threads;
    return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* rays                                                                      */
/* ------------------------------------------------------------------------ */

/* librta/cuda-vec.h:157-193 vector helpers, in the same operation order */
static inline void v_div(float *o, const float *a, float s)
{ o[0] = a[0] / s; o[1] = a[1] / s; o[2] = a[2] / s; }
static inline void v_mul(float *o, const float *a, float s)
{ o[0] = a[0] * s; o[1] = a[1] * s; o[2] = a[2] * s; }
static inline void v_add(float *o, const float *a, const float *b)
{ o[0] = a[0] + b[0]; o[1] = a[1] + b[1]; o[2] = a[2] + b[2]; }
static inline float v_dot(const float *a, const float *b)
{ float s = a[0] * b[0]; s = s + a[1] * b[1]; s = s + a[2] * b[2]; return s; }
static inline float v_len(const float *a) { return sqrtf(v_dot(a, a)); }
static inline void v_cross(float *o, const float *l, const float *r)
{
    float x = (l[1] * r[2]) - (l[2] * r[1]);
    float y = (l[2] * r[0]) - (l[0] * r[2]);
    float z = (l[0] * r[1]) - (l[1] * r[0]);
    o[0] = x; o[1] = y; o[2] = z;
}

void orc_shirley_rays(float *dirs, float *orgs, float *maxts, float height, float aspect,
                      int w, int h, const float vd[3], const float pos[3], const float up[3],
                      float maxt)
{
    /* setup_shirley_rays, cuda-kernels.cu:50-112 */
    const float width = aspect * height;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            size_t id = (size_t)y * w + x;
            orgs[3 * id + 0] = pos[0];
            orgs[3 * id + 1] = pos[1];
            orgs[3 * id + 2] = pos[2];
            maxts[id] = maxt;
            float u_s = (((float)x + 0.5f) / (float)w) * 2.0f - 1.0f;
            float v_s = (((float)y + 0.5f) / (float)h) * 2.0f - 1.0f;
            u_s = width * u_s;
            v_s = height * v_s;
            float W[3], TxW[3], U[3], V[3];
            v_div(W, vd, v_len(vd));
            v_cross(TxW, up, W);
            v_div(U, TxW, v_len(TxW));
            v_cross(V, W, U);
            float dir[3], tmp[3];
            v_mul(dir, U, u_s);
            v_mul(tmp, V, v_s);
            v_add(dir, dir, tmp);
            v_add(dir, dir, W);
            float len = v_len(dir);
            v_div(dir, dir, len);
            dirs[3 * id + 0] = dir[0];
            dirs[3 * id + 1] = dir[1];
            dirs[3 * id + 2] = dir[2];
        }
}

void orc_reset_hits(orc_hit *hits, uint32_t n)
{
    /* reset_intersections, cuda-kernels.cu:24-30 (ref is left alone) */
    for (uint32_t i = 0; i < n; ++i) {
        hits[i].t = FLT_MAX;
        hits[i].beta = 1;
        hits[i].gamma = 2;
    }
}

/* ---- added diffuse bounce (no reference counterpart) ---- */

/* 32-bit integer finaliser (a "lowbias32"-style xor-shift-multiply hash) */
static inline uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

float orc_uniform(uint32_t seed, uint32_t index)
{
    uint32_t h = hash32(index * 0x9e3779b1u + hash32(seed ^ 0x5bd1e995u));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

void orc_cos_sin_2pi(float u, float *c, float *s)
{
    /* quarter-turn reduction, then Taylor polynomials of sin and cos on
     * [0, pi/2) evaluated in Horner form with fused multiply-adds.  Every
     * step is an IEEE operation, so CPU and GPU give the same bits.        */
    float u4 = u * 4.0f;
    int q = (int)u4;
    if (q > 3) q = 3;
    float f = u4 - (float)q;
    float th = f * 1.57079637f;
    float x2 = th * th;
    float sp = -2.50521084e-08f;                 /* -1/11! */
    sp = fmaf(sp, x2, 2.75573192e-06f);          /* 1/9!   */
    sp = fmaf(sp, x2, -1.98412698e-04f);         /* -1/7!  */
    sp = fmaf(sp, x2, 8.33333333e-03f);          /* 1/5!   */
    sp = fmaf(sp, x2, -1.66666667e-01f);         /* -1/3!  */
    sp = fmaf(sp, x2, 1.0f);
    float sn = sp * th;
    float cp = 2.08767570e-09f;                  /* 1/12!  */
    cp = fmaf(cp, x2, -2.75573192e-07f);         /* -1/10! */
    cp = fmaf(cp, x2, 2.48015873e-05f);          /* 1/8!   */
    cp = fmaf(cp, x2, -1.38888889e-03f);         /* -1/6!  */
    cp = fmaf(cp, x2, 4.16666667e-02f);          /* 1/4!   */
    cp = fmaf(cp, x2, -0.5f);                    /* -1/2!  */
    float cs = fmaf(cp, x2, 1.0f);
    switch (q) {
    case 0: *c = cs; *s = sn; break;
    case 1: *c = -sn; *s = cs; break;
    case 2: *c = -cs; *s = -sn; break;
    default: *c = sn; *s = -cs; break;
    }
}

uint32_t orc_diffuse_bounce(const float *tris, const float *orig, const float *dir,
                            const orc_hit *hits, uint32_t nrays, uint32_t seed, float eps,
                            float *oo, float *od, float *om, uint32_t *osrc)
{
    uint32_t m = 0;
    for (uint32_t i = 0; i < nrays; ++i) {
        if (hits[i].t == FLT_MAX) continue;
        const float *tr = tris + (size_t)hits[i].ref * TRI;
        const float *o = orig + 3 * (size_t)i, *d = dir + 3 * (size_t)i;
        float t = hits[i].t;
        float p[3], e1[3], e2[3], nrm[3];
        for (int k = 0; k < 3; ++k) {
            float td = t * d[k];
            p[k] = o[k] + td;
            e1[k] = tr[3 + k] - tr[k];
            e2[k] = tr[6 + k] - tr[k];
        }
        v_cross(nrm, e1, e2);
        float len = v_len(nrm);
        v_div(nrm, nrm, len);
        if (v_dot(nrm, d) > 0.0f) { nrm[0] = -nrm[0]; nrm[1] = -nrm[1]; nrm[2] = -nrm[2]; }
        float u1 = orc_uniform(seed, 2u * i), u2 = orc_uniform(seed, 2u * i + 1u);
        float r = sqrtf(u1);
        float cs, sn;
        orc_cos_sin_2pi(u2, &cs, &sn);
        float lx = r * cs, ly = r * sn;
        float one_m = 1.0f - u1;
        float lz = sqrtf(one_m > 0.0f ? one_m : 0.0f);
        /* orthonormal basis around nrm: Duff et al., "Building an Orthonormal
         * Basis, Revisited", JCGT 6(1), 2017 */
        float sgn = copysignf(1.0f, nrm[2]);
        float a = -1.0f / (sgn + nrm[2]);
        float b = nrm[0] * nrm[1] * a;
        float b1[3] = {1.0f + sgn * nrm[0] * nrm[0] * a, sgn * b, -sgn * nrm[0]};
        float b2[3] = {b, sgn + nrm[1] * nrm[1] * a, -nrm[1]};
        for (int k = 0; k < 3; ++k) {
            float v = b1[k] * lx;
            v = v + b2[k] * ly;
            v = v + nrm[k] * lz;
            od[3 * (size_t)m + k] = v;
            float off = nrm[k] * eps;
            oo[3 * (size_t)m + k] = p[k] + off;
        }
        om[m] = FLT_MAX;
        if (osrc) osrc[m] = i;
        ++m;
    }
    return m;
}

/* ------------------------------------------------------------------------ */
/* CPU bbvh plugin restatement (bbvh/bbvh.h)                                 */
/* ------------------------------------------------------------------------ */

/* center_of_gravity (librta/tri.h:8-14): float sum times the double 0.33333 */
static inline float cog_comp(const float *t, int k)
{
    float s = t[k] + t[3 + k];
    s = s + t[6 + k];
    return (float)((double)s * 0.33333);
}

static int cmp_x(const void *a, const void *b)
{
    float ca = cog_comp((const float *)a, 0), cb = cog_comp((const float *)b, 0);
    if (ca < cb) return -1;
    else if (ca == cb) return 0;
    return 1;
}
static int cmp_y(const void *a, const void *b)
{
    float ca = cog_comp((const float *)a, 1), cb = cog_comp((const float *)b, 1);
    if (ca < cb) return -1;
    else if (ca == cb) return 0;
    return 1;
}
static int cmp_z(const void *a, const void *b)
{
    float ca = cog_comp((const float *)a, 2), cb = cog_comp((const float *)b, 2);
    if (ca < cb) return -1;
    else if (ca == cb) return 0;
    return 1;
}

typedef struct {
    float *tris;
    float *out_tris;
    uint32_t out_n;
    float *nodes;
    uint32_t n_nodes, max_nodes;
    int fail;
} bbvh_ctx;

static uint32_t bbvh_build_sm(bbvh_ctx *cx, uint32_t begin, uint32_t end)
{
    /* build_sm, bbvh.h:206-248 */
    if (cx->n_nodes >= cx->max_nodes) { cx->fail = 1; return 0; }
    uint32_t id = cx->n_nodes++;
    float *nd = cx->nodes + (size_t)id * NODE;
    memset(nd, 0, NODE * sizeof(float));
    float *T = cx->tris;
    /* compute_aabb (aabb.h:109-118) with merge (:79-96) */
    float mn[3], mx[3];
    for (int k = 0; k < 3; ++k) mn[k] = mx[k] = T[(size_t)begin * TRI + k];
    for (uint32_t it = begin; it != end; ++it)
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) {
                float x = T[(size_t)it * TRI + 3 * v + k];
                if (x < mn[k]) mn[k] = x;
                if (x > mx[k]) mx[k] = x;
            }
    for (int k = 0; k < 3; ++k) { nd[2 + k] = mn[k]; nd[5 + k] = mx[k]; }
    uint32_t elems = end - begin;
    if (elems > 4) {
        float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        int axis;
        if (dx > dy) axis = (dx > dz) ? 0 : 2;
        else axis = (dy > dz) ? 1 : 2;
        int (*cmp)(const void *, const void *) = axis == 0 ? cmp_x : axis == 1 ? cmp_y : cmp_z;
        qsort(T + (size_t)begin * TRI, elems, TRI * sizeof(float), cmp);
        /* compute_spatial_median, bbvh.h:187-204 */
        float min_cog = cog_comp(T + (size_t)begin * TRI, axis), max_cog = min_cog;
        for (uint32_t it = begin; it != end; ++it) {
            float tmp = cog_comp(T + (size_t)it * TRI, axis);
            if (tmp < min_cog) min_cog = tmp;
            if (tmp > max_cog) max_cog = tmp;
        }
        float s = (max_cog - min_cog) / 2 + min_cog;
        uint32_t mid = begin;
        while (mid != end && cog_comp(T + (size_t)mid * TRI, axis) < s) ++mid;
        if (begin == mid || mid == end) mid = begin + (end - begin) / 2;
        uint32_t left = bbvh_build_sm(cx, begin, mid);
        uint32_t right = bbvh_build_sm(cx, mid, end);
        nd = cx->nodes + (size_t)id * NODE;
        node_set_inner(nd, left, right);
    } else {
        uint32_t idx = cx->out_n;
        for (uint32_t i = 0; i < elems; ++i)
            memcpy(cx->out_tris + (size_t)(cx->out_n++) * TRI, T + (size_t)(begin + i) * TRI,
                   TRI * sizeof(float));
        node_set_leaf(nd, idx, elems);
    }
    return id;
}

int64_t orc_bbvh_build(float *tris, uint32_t n, float *out_tris, float *nodes, uint32_t max_nodes)
{
    if (n == 0) return -1;
    bbvh_ctx cx = {tris, out_tris, 0, nodes, 0, max_nodes, 0};
    bbvh_build_sm(&cx, 0, n);
    if (cx.fail) return -2;
    return (int64_t)cx.n_nodes;
}

static void bbvh_trace_one(const float *nodes, const float *tris, const float *o,
                           const float *dir, float max_t, orc_hit *out)
{
    /* bbvh_child_is_tracer::trace_ray, bbvh.h:407-455 (stack of 128,
     * raytrav.h:24) */
    uint32_t stack[128];
    int sp = 0;
    stack[0] = 0;
    orc_hit best;
    best.t = max_t;
    best.ref = 0;
    best.beta = 0;
    best.gamma = 0;
    while (sp >= 0) {
        uint32_t node = stack[sp--];
        const float *cur = nodes + (size_t)node * NODE;
        if (node_inner(cur)) {
            float dl = 0, dr = 0, mn[3], mx[3];
            uint32_t nl = node_left(cur), nr = node_right(cur);
            node_box(nodes, nl, mn, mx);
            int do_l = orc_intersect_aabb(mn, mx, o, dir, &dl);
            node_box(nodes, nr, mn, mx);
            int do_r = orc_intersect_aabb(mn, mx, o, dir, &dr);
            do_l = do_l && dl < best.t && dl <= max_t;
            do_r = do_r && dr < best.t && dr <= max_t;
            if (sp + 2 >= 128) break;
            if (do_l && do_r) {
                if (dl <= dr) { stack[++sp] = nr; stack[++sp] = nl; }
                else { stack[++sp] = nl; stack[++sp] = nr; }
            } else if (do_l)
                stack[++sp] = nl;
            else if (do_r)
                stack[++sp] = nr;
        } else {
            uint32_t elems = f_bits(cur[0]) >> 1, offset = f_bits(cur[1]);
            for (uint32_t i = 0; i < elems; ++i) {
                float t, b, g;
                if (orc_intersect_tri(tris + (size_t)(offset + i) * TRI, o, dir, &t, &b, &g))
                    if (t < best.t && t <= max_t) {
                        best.t = t;
                        best.beta = b;
                        best.gamma = g;
                        best.ref = offset + i;
                    }
            }
        }
    }
    *out = best;
}

int orc_bbvh_trace_cis(const float *nodes, const float *tris, const float *orig,
                       const float *dir, const float *maxt, uint32_t nrays, orc_hit *hits,
                       int threads)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 32) num_threads(threads)
#endif
    for (long long i = 0; i < (long long)nrays; ++i)
        bbvh_trace_one(nodes, tris, orig + 3 * i, dir + 3 * i, maxt[i], hits + i);
    (void)threads;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* host shading                                                               */
/* ------------------------------------------------------------------------- */

/* the conversions of lighting_collector: int(x*255) truncates toward zero */
static int orc_to_int255(float x)
{
    const float v = x * 255.0f;
    if (!(v == v)) return 0;
    if (v >= 2147483647.0f) return 2147483647;
    if (v <= -2147483648.0f) return (int)0x80000000u;
    return (int)v;
}

/* barycentric_interpolation (librta/tri.h:41-48): a*b0 + b*b1, then + c*b2 */
static void orc_bary(float out[3], const float bc[3], const float *a, const float *b, const float *c)
{
    for (int k = 0; k < 3; ++k) {
        float to = a[k] * bc[0];
        float tmp = b[k] * bc[1];
        to = to + tmp;
        tmp = c[k] * bc[2];
        out[k] = to + tmp;
    }
}

static float orc_dot3(const float *l, const float *r)
{
    float s = l[0] * r[0];
    s = s + l[1] * r[1];
    s = s + l[2] * r[2];
    return s;
}

/* normalize_vec3f (librta/cuda-vec.h:183-188): v / sqrtf(dot(v, v)) */
static void orc_normalize3(float v[3])
{
    const float len = sqrtf(orc_dot3(v, v));
    for (int k = 0; k < 3; ++k) v[k] = v[k] / len;
}

void orc_shade_lambert(const float *tris, const orc_hit *hits, uint32_t w, uint32_t h,
                       const float *lights, uint32_t nl, int binary, const float *bg,
                       uint8_t *img)
{
    const size_t n = (size_t)w * h;
    if (bg) {
        /* reset (raytrav.h:189-194): min(int(c*255), 255) stored as a byte */
        for (size_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                int v = orc_to_int255(bg[k]);
                img[3 * i + k] = (uint8_t)(v < 255 ? v : 255);
            }
    }
    if (nl == 0) return;
    for (size_t i = 0; i < n; ++i) {
        const orc_hit *is = &hits[i];
        if (is->t == FLT_MAX) continue;
        float col[3] = {0.0f, 0.0f, 0.0f};
        if (binary) {
            col[0] = lights[3];
            col[1] = lights[4];
            col[2] = lights[5];
        } else {
            const float *tri = tris + (size_t)is->ref * 26;
            for (uint32_t l = 0; l < nl; ++l) {
                const float *L0 = lights + 6 * l;
                /* triangle_intersection::barycentric_coord (basic_types.h:90-94):
                   x = 1.0 - beta - gamma in double, stored as float */
                const float bc[3] = {(float)(1.0 - (double)is->beta - (double)is->gamma), is->beta, is->gamma};
                float N[3], p[3];
                orc_bary(N, bc, tri + 9, tri + 12, tri + 15);
                orc_bary(p, bc, tri + 0, tri + 3, tri + 6);
                float L[3] = {L0[0] - p[0], L0[1] - p[1], L0[2] - p[2]};
                orc_normalize3(L);
                orc_normalize3(N);
                float dot = orc_dot3(N, L);
                dot = (dot < 0.0f) ? 0.0f : dot;   /* std::max(dot, 0) */
                for (int k = 0; k < 3; ++k) col[k] = col[k] + L0[3 + k] * dot;
            }
        }
        for (int k = 0; k < 3; ++k) {
            int v = orc_to_int255(col[k]);
            v = v < 255 ? v : 255;
            img[3 * i + k] = (uint8_t)(v > 0 ? v : 0);
        }
    }
}
