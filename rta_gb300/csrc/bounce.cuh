// bounce.cuh -- the diffuse bounce ray of one primary hit, shared by the
// bounce pass (k_bounce, rays.cu) and the frame kernel that traces each
// bounce ray right after its primary ray (k_trace FUSE, trace.cu): vector
// helpers in the reference's operation order, the seeded uniforms and the
// cosine-weighted direction.  IEEE operations only, so the CPU oracle
// (oracle/oracle.c orc_diffuse_bounce) reproduces every bit.
#pragma once

#include "common.cuh"

namespace rta {

// librta/cuda-vec.h:157-193 in the same operation order
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v_div(V3 a, float s)
{
    return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)};
}
__device__ __forceinline__ V3 v_mul(V3 a, float s)
{
    return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
__device__ __forceinline__ V3 v_add(V3 a, V3 b)
{
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ float v_dot(V3 a, V3 b)
{
    float s = __fmul_rn(a.x, b.x);
    s = __fadd_rn(s, __fmul_rn(a.y, b.y));
    s = __fadd_rn(s, __fmul_rn(a.z, b.z));
    return s;
}
__device__ __forceinline__ float v_len(V3 a) { return __fsqrt_rn(v_dot(a, a)); }
__device__ __forceinline__ V3 v_cross(V3 l, V3 r)
{
    return {__fsub_rn(__fmul_rn(l.y, r.z), __fmul_rn(l.z, r.y)),
            __fsub_rn(__fmul_rn(l.z, r.x), __fmul_rn(l.x, r.z)),
            __fsub_rn(__fmul_rn(l.x, r.y), __fmul_rn(l.y, r.x))};
}


// 32-bit xor-shift-multiply finaliser; the oracle uses the same function
__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float uniform01(uint32_t seed, uint32_t index)
{
    uint32_t h = hash32(index * 0x9e3779b1u + hash32(seed ^ 0x5bd1e995u));
    return __fmul_rn((float)(h >> 8), 1.0f / 16777216.0f);
}

// cos and sin of 2*pi*u: quarter-turn reduction and Taylor polynomials in
// Horner form with fused multiply-adds -- IEEE operations only, so the
// oracle reproduces them bit for bit
__device__ __forceinline__ void cos_sin_2pi(float u, float &c, float &s)
{
    float u4 = __fmul_rn(u, 4.0f);
    int q = (int)u4;
    if (q > 3) q = 3;
    float f = __fsub_rn(u4, (float)q);
    float th = __fmul_rn(f, 1.57079637f);
    float x2 = __fmul_rn(th, th);
    float sp = -2.50521084e-08f;
    sp = __fmaf_rn(sp, x2, 2.75573192e-06f);
    sp = __fmaf_rn(sp, x2, -1.98412698e-04f);
    sp = __fmaf_rn(sp, x2, 8.33333333e-03f);
    sp = __fmaf_rn(sp, x2, -1.66666667e-01f);
    sp = __fmaf_rn(sp, x2, 1.0f);
    float sn = __fmul_rn(sp, th);
    float cp = 2.08767570e-09f;
    cp = __fmaf_rn(cp, x2, -2.75573192e-07f);
    cp = __fmaf_rn(cp, x2, 2.48015873e-05f);
    cp = __fmaf_rn(cp, x2, -1.38888889e-03f);
    cp = __fmaf_rn(cp, x2, 4.16666667e-02f);
    cp = __fmaf_rn(cp, x2, -0.5f);
    float cs = __fmaf_rn(cp, x2, 1.0f);
    switch (q) {
    case 0: c = cs; s = sn; break;
    case 1: c = -sn; s = cs; break;
    case 2: c = -cs; s = -sn; break;
    default: c = sn; s = -cs; break;
    }
}

// One cosine-weighted diffuse bounce ray of primary ray i, which hit
// triangle T at distance t: origin = hit point pushed eps along the geometric
// normal (turned to face the incoming ray), direction from the uniform pair
// (seed, 2i), (seed, 2i+1) in the normal's orthonormal basis.
__device__ __forceinline__ void bounce_ray(const TriRec &T, const float oi[3], const float di[3], float t,
                                           uint32_t i, uint32_t seed, float eps, float bo[3], float bd[3])
{
    const V3 o = {oi[0], oi[1], oi[2]};
    const V3 d = {di[0], di[1], di[2]};
    V3 p = {__fadd_rn(o.x, __fmul_rn(t, d.x)), __fadd_rn(o.y, __fmul_rn(t, d.y)),
            __fadd_rn(o.z, __fmul_rn(t, d.z))};
    V3 e1 = {__fsub_rn(T.v1.x, T.v0.x), __fsub_rn(T.v1.y, T.v0.y), __fsub_rn(T.v1.z, T.v0.z)};
    V3 e2 = {__fsub_rn(T.v2.x, T.v0.x), __fsub_rn(T.v2.y, T.v0.y), __fsub_rn(T.v2.z, T.v0.z)};
    V3 nrm = v_cross(e1, e2);
    nrm = v_div(nrm, v_len(nrm));
    if (v_dot(nrm, d) > 0.0f) nrm = {-nrm.x, -nrm.y, -nrm.z};
    const float u1 = uniform01(seed, 2u * i), u2 = uniform01(seed, 2u * i + 1u);
    const float rr = __fsqrt_rn(u1);
    float cs, sn;
    cos_sin_2pi(u2, cs, sn);
    const float lx = __fmul_rn(rr, cs), ly = __fmul_rn(rr, sn);
    const float one_m = __fsub_rn(1.0f, u1);
    const float lz = __fsqrt_rn(one_m > 0.0f ? one_m : 0.0f);
    // orthonormal basis: Duff et al., JCGT 6(1), 2017
    const float sg = copysignf(1.0f, nrm.z);
    const float a = __fdiv_rn(-1.0f, __fadd_rn(sg, nrm.z));
    const float b = __fmul_rn(__fmul_rn(nrm.x, nrm.y), a);
    const V3 b1 = {__fadd_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(sg, nrm.x), nrm.x), a)),
                   __fmul_rn(sg, b), -__fmul_rn(sg, nrm.x)};
    const V3 b2 = {b, __fadd_rn(sg, __fmul_rn(__fmul_rn(nrm.y, nrm.y), a)), -nrm.y};
    bd[0] = __fadd_rn(__fadd_rn(__fmul_rn(b1.x, lx), __fmul_rn(b2.x, ly)), __fmul_rn(nrm.x, lz));
    bd[1] = __fadd_rn(__fadd_rn(__fmul_rn(b1.y, lx), __fmul_rn(b2.y, ly)), __fmul_rn(nrm.y, lz));
    bd[2] = __fadd_rn(__fadd_rn(__fmul_rn(b1.z, lx), __fmul_rn(b2.z, ly)), __fmul_rn(nrm.z, lz));
    bo[0] = __fadd_rn(p.x, __fmul_rn(nrm.x, eps));
    bo[1] = __fadd_rn(p.y, __fmul_rn(nrm.y, eps));
    bo[2] = __fadd_rn(p.z, __fmul_rn(nrm.z, eps));
}

} // namespace rta
