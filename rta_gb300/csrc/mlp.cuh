// mlp.cuh -- the child-order network: 14 -> 32 -> 32 -> 1, ReLU, BF16 weights
// and activations, FP32 accumulation on the tensor cores (mma.sync m16n8k16).
//
// One warp evaluates 32 rows at once (one row per lane, 16 inputs: 14
// features and two zeros).  Row r of the batch is m-tile r/16, tile row r%16.
// Fragment layouts (PTX ISA, mma.m16n8k16 .bf16):
//   A (16x16, row)  lane holds rows g, g+8 and columns 2t, 2t+1, 8+2t, 8+2t+1
//   B (16x8, col)   lane holds k = 2t, 2t+1, 8+2t, 8+2t+1 of column g
//   C (16x8)        lane holds rows g, g+8 and columns 2t, 2t+1
// with g = lane/4, t = lane%4.  The C fragments of two adjacent n8 tiles are
// exactly the A fragment of the matching k16 slice, so a layer's output feeds
// the next layer without leaving registers.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace rta {

constexpr int kMlpIn = 16;       // 14 features + 2 zero pads
constexpr int kMlpFeatures = 14;
constexpr int kMlpHidden = 32;

// weights the kernels read (bf16, [out][in] row-major), biases in fp32
struct MlpWeights {
    __nv_bfloat16 w1[kMlpHidden][kMlpIn];
    __nv_bfloat16 w2[kMlpHidden][kMlpHidden];
    __nv_bfloat16 w2t[kMlpHidden][kMlpHidden];   // w2 transposed (backward pass)
    __nv_bfloat16 w3[kMlpHidden];
    float b1[kMlpHidden];
    float b2[kMlpHidden];
    float b3;
    float margin;   // the network overrides the plain order only where |logit| > margin
    float pad[2];
};

// one decision of the plain traversal, as recorded for training: the
// features, the ray, the two children's Morton ranges, and (after the ray has
// finished) the label: 1 if the final hit lies under the left child, 0 if
// under the right one; weight 0 when it lies under neither.
struct __align__(16) Sample {
    __nv_bfloat16 x[kMlpIn];
    uint32_t ray;
    uint32_t lfirst, lsize, rfirst, rsize;
    float label, weight;
    uint32_t pad;
};
static_assert(sizeof(Sample) == 64, "sample record");

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p)
{
    return *reinterpret_cast<const uint32_t *>(p);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float relu(float x) { return x > 0.0f ? x : 0.0f; }

// Activations of one warp's forward pass, kept for the backward pass.
struct MlpForward {
    float z1[2][4][4];   // [m-tile][n-tile][c0..c3] pre-activation, layer 1
    float z2[2][4][4];   // layer 2
    float logit_g[2];    // logits of rows g and g+8 of each m-tile (reduced over t)
    float logit_g8[2];
};

// Forward pass.  xs is the warp's 32 x 16 input tile (bf16, shared memory).
__device__ __forceinline__ void mlp_forward(const MlpWeights &W, const __nv_bfloat16 (*xs)[kMlpIn],
                                            MlpForward &F)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int r0 = mt * 16 + g, r1 = r0 + 8;
        uint32_t a[4] = {ld_pair(&xs[r0][2 * t]), ld_pair(&xs[r1][2 * t]), ld_pair(&xs[r0][8 + 2 * t]),
                         ld_pair(&xs[r1][8 + 2 * t])};
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int n = nt * 8;
            uint32_t b[2] = {ld_pair(&W.w1[n + g][2 * t]), ld_pair(&W.w1[n + g][8 + 2 * t])};
            float *c = F.z1[mt][nt];
            c[0] = c[2] = W.b1[n + 2 * t];
            c[1] = c[3] = W.b1[n + 2 * t + 1];
            mma_bf16(c, a, b);
        }
        // layer 2: the ReLU'd layer-1 tiles are the A fragments of its two k16 slices
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int n = nt * 8;
            float *c = F.z2[mt][nt];
            c[0] = c[2] = W.b2[n + 2 * t];
            c[1] = c[3] = W.b2[n + 2 * t + 1];
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                const float *lo = F.z1[mt][2 * kt], *hi = F.z1[mt][2 * kt + 1];
                uint32_t ah[4] = {pack_bf16(relu(lo[0]), relu(lo[1])), pack_bf16(relu(lo[2]), relu(lo[3])),
                                  pack_bf16(relu(hi[0]), relu(hi[1])), pack_bf16(relu(hi[2]), relu(hi[3]))};
                uint32_t b[2] = {ld_pair(&W.w2[n + g][kt * 16 + 2 * t]),
                                 ld_pair(&W.w2[n + g][kt * 16 + 8 + 2 * t])};
                mma_bf16(c, ah, b);
            }
        }
        // layer 3 (32 -> 1): bf16 activations times bf16 weights, fp32 sums
        float sg = 0.0f, sg8 = 0.0f;
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const float w = __bfloat162float(W.w3[nt * 8 + 2 * t + j]);
                sg += __bfloat162float(__float2bfloat16_rn(relu(F.z2[mt][nt][j]))) * w;
                sg8 += __bfloat162float(__float2bfloat16_rn(relu(F.z2[mt][nt][2 + j]))) * w;
            }
        sg += __shfl_xor_sync(0xffffffffu, sg, 1);
        sg += __shfl_xor_sync(0xffffffffu, sg, 2);
        sg8 += __shfl_xor_sync(0xffffffffu, sg8, 1);
        sg8 += __shfl_xor_sync(0xffffffffu, sg8, 2);
        F.logit_g[mt] = sg + W.b3;
        F.logit_g8[mt] = sg8 + W.b3;
    }
}

// The logit of this lane's own row (row = lane).
__device__ __forceinline__ float mlp_own_logit(const MlpForward &F)
{
    const int lane = threadIdx.x & 31;
    const int mt = lane >> 4, rr = lane & 15, src = (rr & 7) * 4;
    const float v0 = __shfl_sync(0xffffffffu, F.logit_g[0], src);
    const float v1 = __shfl_sync(0xffffffffu, F.logit_g8[0], src);
    const float v2 = __shfl_sync(0xffffffffu, F.logit_g[1], src);
    const float v3 = __shfl_sync(0xffffffffu, F.logit_g8[1], src);
    return mt == 0 ? (rr < 8 ? v0 : v1) : (rr < 8 ? v2 : v3);
}

} // namespace rta
