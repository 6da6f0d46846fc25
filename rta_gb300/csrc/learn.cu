// learn.cu -- training of the child-order network on the tensor cores.
//
// Samples come from the plain child-is traversal (k_trace_learn in trace.cu
// records one per node where both children are hit and not culled); the
// label says which child's subtree holds the ray's final closest hit.  The
// network (mlp.cuh) is trained with binary cross-entropy and Adam:
//   k_label     label + weight of each sample from the final hits (weight =
//               bit length of the other child's triangle count)
//   k_mlp_grad  forward and backward of 32-row tiles per warp, every product
//               on mma.sync bf16 with fp32 accumulation; weight gradients
//               accumulate in registers across tiles, then per block in shared
//               memory, then once per block into a partial-sum row, which
//               k_grad_reduce adds up (no atomics on the 1633 gradients)
//   k_adam      Adam step on the fp32 master weights, republishes the bf16
//               weights the kernels read
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "mlp.cuh"

namespace rta {

constexpr int kParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden +
                        kMlpHidden + 1;   // 1633
// offsets of the flat fp32 parameter / gradient vector
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHidden * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden;

// ---- labels ---- //

// labels samples [begin, min(count, cap)) from the hits of the batch that made them
__global__ void k_label(Sample *__restrict__ s, const uint32_t *__restrict__ d_count, uint32_t cap,
                        uint32_t begin, const HitRec *__restrict__ hits)
{
    const uint32_t n = min(*d_count, cap);
    for (uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Sample &x = s[i];
        const HitRec h = hits[x.ray];
        // the weight is the size class (bit length of the triangle count) of
        // the subtree a wrong first choice would enter: a mistake costs about
        // the depth of that subtree
        float label = 0.f, weight = 0.f;
        if (h.t != FLT_MAX) {
            if (h.ref - x.lfirst < x.lsize) { label = 1.f; weight = (float)(32 - __clz(x.rsize)); }
            else if (h.ref - x.rfirst < x.rsize) { label = 0.f; weight = (float)(32 - __clz(x.lsize)); }
        }
        x.label = label;
        x.weight = weight;
    }
}

// ---- forward + backward ---- //

constexpr int kGradWarps = 4;

struct GradSmem {
    MlpWeights w;
    __nv_bfloat16 xs[kGradWarps][32][kMlpIn];
    __nv_bfloat16 xt[kGradWarps][kMlpIn][32];
    __nv_bfloat16 h1t[kGradWarps][kMlpHidden][32];
    __nv_bfloat16 dz2t[kGradWarps][kMlpHidden][32];
    __nv_bfloat16 dz1t[kGradWarps][kMlpHidden][32];
    float grad[kParams];
    float loss;
};

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Gradient of the mean binary cross-entropy (logits vs labels, per-sample
// weights) over rows [first, first+count) of `samples`, scaled by `scale`,
// added into grad[kParams]; the weighted loss sum is added into *loss.
// Each block writes its sums to partial[block * (kParams + 1) ...] (the
// loss last); k_grad_reduce adds the blocks' sums into the gradient.
__global__ void __launch_bounds__(kGradWarps * 32)
k_mlp_grad(const MlpWeights *__restrict__ wg, const Sample *__restrict__ samples, uint32_t first,
           uint32_t count, float scale, float *__restrict__ partial)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GradSmem &S = *reinterpret_cast<GradSmem *>(smem_raw);
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(wg);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&S.w);
        for (int i = tid; i < (int)(sizeof(MlpWeights) / 4); i += blockDim.x) dst[i] = src[i];
        for (int i = tid; i < kParams; i += blockDim.x) S.grad[i] = 0.f;
        if (tid == 0) S.loss = 0.f;
    }
    __syncthreads();
    const MlpWeights &W = S.w;

    float dw2[2][4][4] = {}, dw1[2][2][4] = {};
    float db1[4][2] = {}, db2[4][2] = {}, dw3[4][2] = {};
    float db3 = 0.f, lsum = 0.f;

    const uint32_t tiles = (count + 31) / 32;
    const uint32_t gw = blockIdx.x * kGradWarps + w, nw = gridDim.x * kGradWarps;
    for (uint32_t tile = gw; tile < tiles; tile += nw) {
        const uint32_t row = tile * 32 + lane;
        const bool valid = row < count;
        float label = 0.f, weight = 0.f;
        uint4 x0 = make_uint4(0, 0, 0, 0), x1 = x0;
        if (valid) {
            const Sample &s = samples[first + row];
            x0 = *reinterpret_cast<const uint4 *>(&s.x[0]);
            x1 = *reinterpret_cast<const uint4 *>(&s.x[8]);
            label = s.label;
            weight = s.weight;
        }
        *reinterpret_cast<uint4 *>(&S.xs[w][lane][0]) = x0;
        *reinterpret_cast<uint4 *>(&S.xs[w][lane][8]) = x1;
        __syncwarp();
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) S.xt[w][k][lane] = S.xs[w][lane][k];
        MlpForward F;
        mlp_forward(W, S.xs[w], F);
        const float y = mlp_own_logit(F);
        // d(mean BCE)/dy = sigmoid(y) - label
        const float p = 1.0f / (1.0f + __expf(-y));
        const float dy = (p - label) * weight * scale;
        lsum += weight * (fmaxf(y, 0.f) - y * label + log1pf(__expf(-fabsf(y))));
        db3 += dy;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const float dyg = __shfl_sync(0xffffffffu, dy, mt * 16 + g);
            const float dyg8 = __shfl_sync(0xffffffffu, dy, mt * 16 + g + 8);
            const int r0 = mt * 16 + g, r1 = r0 + 8;
            float dz2[4][4];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int col = nt * 8 + 2 * t + j;
                    const float w3 = __bfloat162float(W.w3[col]);
                    const float z2a = F.z2[mt][nt][j], z2b = F.z2[mt][nt][2 + j];
                    dw3[nt][j] += dyg * bf(relu(z2a)) + dyg8 * bf(relu(z2b));
                    dz2[nt][j] = z2a > 0.f ? dyg * w3 : 0.f;
                    dz2[nt][2 + j] = z2b > 0.f ? dyg8 * w3 : 0.f;
                    db2[nt][j] += dz2[nt][j] + dz2[nt][2 + j];
                    S.dz2t[w][col][r0] = __float2bfloat16_rn(dz2[nt][j]);
                    S.dz2t[w][col][r1] = __float2bfloat16_rn(dz2[nt][2 + j]);
                    S.h1t[w][col][r0] = __float2bfloat16_rn(relu(F.z1[mt][nt][j]));
                    S.h1t[w][col][r1] = __float2bfloat16_rn(relu(F.z1[mt][nt][2 + j]));
                }
            // dh1 = dz2 . W2 : the dz2 tiles are A fragments, W2^T rows are B columns
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                float dh1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int kt = 0; kt < 2; ++kt) {
                    const float *lo = dz2[2 * kt], *hi = dz2[2 * kt + 1];
                    uint32_t a[4] = {pack_bf16(lo[0], lo[1]), pack_bf16(lo[2], lo[3]), pack_bf16(hi[0], hi[1]),
                                     pack_bf16(hi[2], hi[3])};
                    uint32_t b[2] = {ld_pair(&W.w2t[nt * 8 + g][kt * 16 + 2 * t]),
                                     ld_pair(&W.w2t[nt * 8 + g][kt * 16 + 8 + 2 * t])};
                    mma_bf16(dh1, a, b);
                }
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int col = nt * 8 + 2 * t + j;
                    const float za = F.z1[mt][nt][j], zb = F.z1[mt][nt][2 + j];
                    const float da = za > 0.f ? dh1[j] : 0.f, dbv = zb > 0.f ? dh1[2 + j] : 0.f;
                    db1[nt][j] += da + dbv;
                    S.dz1t[w][col][r0] = __float2bfloat16_rn(da);
                    S.dz1t[w][col][r1] = __float2bfloat16_rn(dbv);
                }
            }
        }
        __syncwarp();
        // dW2 += dz2^T . h1 and dW1 += dz1^T . x, both reducing over the 32 rows
#pragma unroll
        for (int mo = 0; mo < 2; ++mo)
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                const int o0 = mo * 16 + g, o1 = o0 + 8, k0 = kt * 16 + 2 * t;
                uint32_t a2[4] = {ld_pair(&S.dz2t[w][o0][k0]), ld_pair(&S.dz2t[w][o1][k0]),
                                  ld_pair(&S.dz2t[w][o0][k0 + 8]), ld_pair(&S.dz2t[w][o1][k0 + 8])};
                uint32_t a1[4] = {ld_pair(&S.dz1t[w][o0][k0]), ld_pair(&S.dz1t[w][o1][k0]),
                                  ld_pair(&S.dz1t[w][o0][k0 + 8]), ld_pair(&S.dz1t[w][o1][k0 + 8])};
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) {
                    uint32_t b[2] = {ld_pair(&S.h1t[w][ni * 8 + g][k0]), ld_pair(&S.h1t[w][ni * 8 + g][k0 + 8])};
                    mma_bf16(dw2[mo][ni], a2, b);
                }
#pragma unroll
                for (int ni = 0; ni < 2; ++ni) {
                    uint32_t b[2] = {ld_pair(&S.xt[w][ni * 8 + g][k0]), ld_pair(&S.xt[w][ni * 8 + g][k0 + 8])};
                    mma_bf16(dw1[mo][ni], a1, b);
                }
            }
        __syncwarp();
    }

    // column partials of the biases and w3: sum over the 8 row groups
#pragma unroll
    for (int off = 4; off < 32; off <<= 1)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                db1[nt][j] += __shfl_xor_sync(0xffffffffu, db1[nt][j], off);
                db2[nt][j] += __shfl_xor_sync(0xffffffffu, db2[nt][j], off);
                dw3[nt][j] += __shfl_xor_sync(0xffffffffu, dw3[nt][j], off);
            }
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        db3 += __shfl_xor_sync(0xffffffffu, db3, off);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    }
    if (g == 0)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int col = nt * 8 + 2 * t + j;
                atomicAdd(&S.grad[kOffB1 + col], db1[nt][j]);
                atomicAdd(&S.grad[kOffB2 + col], db2[nt][j]);
                atomicAdd(&S.grad[kOffW3 + col], dw3[nt][j]);
            }
    if (lane == 0) {
        atomicAdd(&S.grad[kOffB3], db3);
        atomicAdd(&S.loss, lsum);
    }
#pragma unroll
    for (int mo = 0; mo < 2; ++mo) {
        const int o0 = mo * 16 + g, o1 = o0 + 8;
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int in = ni * 8 + 2 * t + j;
                atomicAdd(&S.grad[kOffW2 + o0 * kMlpHidden + in], dw2[mo][ni][j]);
                atomicAdd(&S.grad[kOffW2 + o1 * kMlpHidden + in], dw2[mo][ni][2 + j]);
            }
#pragma unroll
        for (int ni = 0; ni < 2; ++ni)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int in = ni * 8 + 2 * t + j;
                atomicAdd(&S.grad[kOffW1 + o0 * kMlpIn + in], dw1[mo][ni][j]);
                atomicAdd(&S.grad[kOffW1 + o1 * kMlpIn + in], dw1[mo][ni][2 + j]);
            }
    }
    __syncthreads();
    float *out = partial + (size_t)blockIdx.x * (kParams + 1);
    for (int i = tid; i < kParams; i += blockDim.x) out[i] = S.grad[i];
    if (tid == 0) out[kParams] = S.loss;
}

// grad[i] += the blocks' partial sums (i = kParams: the loss)
__global__ void k_grad_reduce(const float *__restrict__ partial, uint32_t blocks, float *__restrict__ grad,
                              float *__restrict__ loss)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > (uint32_t)kParams) return;
    float sum = 0.f;
    for (uint32_t b = 0; b < blocks; ++b) sum += partial[(size_t)b * (kParams + 1) + i];
    if (i < (uint32_t)kParams) grad[i] += sum;
    else *loss += sum;
}

constexpr uint32_t kGradMaxBlocks = 1024;

// ---- Adam + publishing the bf16 weights ---- //

__global__ void k_publish(const float *__restrict__ p, MlpWeights *__restrict__ out)
{
    for (int i = threadIdx.x; i < kMlpHidden * kMlpIn; i += blockDim.x)
        out->w1[i / kMlpIn][i % kMlpIn] = __float2bfloat16_rn(p[kOffW1 + i]);
    for (int i = threadIdx.x; i < kMlpHidden * kMlpHidden; i += blockDim.x) {
        const int o = i / kMlpHidden, in = i % kMlpHidden;
        const __nv_bfloat16 v = __float2bfloat16_rn(p[kOffW2 + i]);
        out->w2[o][in] = v;
        out->w2t[in][o] = v;
    }
    for (int i = threadIdx.x; i < kMlpHidden; i += blockDim.x) {
        out->w3[i] = __float2bfloat16_rn(p[kOffW3 + i]);
        out->b1[i] = p[kOffB1 + i];
        out->b2[i] = p[kOffB2 + i];
    }
    if (threadIdx.x == 0) out->b3 = p[kOffB3];
}

__global__ void k_adam(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                       float *__restrict__ grad, float lr, float b1, float b2, float c1, float c2,
                       float eps, MlpWeights *__restrict__ out)
{
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
        const float gr = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        grad[i] = 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kMlpHidden * kMlpIn; i += blockDim.x)
        out->w1[i / kMlpIn][i % kMlpIn] = __float2bfloat16_rn(p[kOffW1 + i]);
    for (int i = threadIdx.x; i < kMlpHidden * kMlpHidden; i += blockDim.x) {
        const int o = i / kMlpHidden, in = i % kMlpHidden;
        const __nv_bfloat16 val = __float2bfloat16_rn(p[kOffW2 + i]);
        out->w2[o][in] = val;
        out->w2t[in][o] = val;
    }
    for (int i = threadIdx.x; i < kMlpHidden; i += blockDim.x) {
        out->w3[i] = __float2bfloat16_rn(p[kOffW3 + i]);
        out->b1[i] = p[kOffB1 + i];
        out->b2[i] = p[kOffB2 + i];
    }
    if (threadIdx.x == 0) out->b3 = p[kOffB3];
}

int trace_impl(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt, uint32_t nrays,
               const uint32_t *d_nrays, void *hits, uint32_t mode, uint32_t *stats, uint32_t *queue, cudaStream_t s);
int trace_learn_impl(const rta_lbvh *bvh, const MlpWeights *w, const float *orig, const float *dir,
                     const float *maxt, uint32_t nrays, const uint32_t *d_nrays, void *hits,
                     uint32_t *stats, Sample *samples, uint32_t *sample_count, uint32_t sample_cap,
                     uint32_t *queue, bool learned, cudaStream_t s, const void *hint = nullptr);

} // namespace rta

using namespace rta;

struct rta_order_model {
    uint32_t cap = 0;
    float margin = 0.0f;   // host copy of MlpWeights::margin
    Sample *samples = nullptr;
    uint32_t *counters = nullptr;   // [0] samples written, [1] trace queue
    float *params = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr;
    float *partial = nullptr;   // per-block gradient sums of k_mlp_grad
    MlpWeights *weights = nullptr;
    int step = 0;
    uint32_t seed = 0;
};

static uint32_t host_hash(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

extern "C" {

uint32_t rta_order_param_count(void) { return kParams; }

int rta_order_create(rta_order_model **out, uint32_t max_samples, uint32_t seed)
{
    if (!out) return RTA_ERR_INVALID;
    rta_order_model *c = new rta_order_model();
    c->cap = max_samples;
    c->seed = seed;
    cudaError_t e = cudaSuccess;
    if (max_samples) e = cudaMalloc(&c->samples, (size_t)max_samples * sizeof(Sample));
    if (e == cudaSuccess) e = cudaMalloc(&c->counters, 16);
    if (e == cudaSuccess) e = cudaMemset(c->counters, 0, 16);
    if (e == cudaSuccess) e = cudaMalloc(&c->params, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->m, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->v, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->grad, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->partial, (size_t)kGradMaxBlocks * (kParams + 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->loss, 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->weights, sizeof(MlpWeights));
    if (e == cudaSuccess) e = cudaMemset(c->m, 0, kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(c->v, 0, kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(c->grad, 0, kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(c->weights, 0, sizeof(MlpWeights));
    if (e != cudaSuccess) {
        set_cuda_error(e, "rta_order_create");
        rta_order_destroy(c);
        return e == cudaErrorMemoryAllocation ? RTA_ERR_NOMEM : RTA_ERR_CUDA;
    }
    // Glorot-uniform weights from a seeded hash, zero biases
    std::vector<float> p(kParams, 0.f);
    auto uni = [&](uint32_t i) {
        return (float)(host_hash(i * 0x9e3779b1u + host_hash(seed)) >> 8) * (1.0f / 16777216.0f) * 2.f - 1.f;
    };
    const float a1 = std::sqrt(6.f / (kMlpFeatures + kMlpHidden)), a2 = std::sqrt(6.f / (2 * kMlpHidden)),
                a3 = std::sqrt(6.f / (kMlpHidden + 1));
    for (int o = 0; o < kMlpHidden; ++o)
        for (int i = 0; i < kMlpIn; ++i)
            p[kOffW1 + o * kMlpIn + i] = i < kMlpFeatures ? a1 * uni(kOffW1 + o * kMlpIn + i) : 0.f;
    for (int i = 0; i < kMlpHidden * kMlpHidden; ++i) p[kOffW2 + i] = a2 * uni(kOffW2 + i);
    for (int i = 0; i < kMlpHidden; ++i) p[kOffW3 + i] = a3 * uni(kOffW3 + i);
    *out = c;
    return rta_order_set_params(c, p.data());
}

int rta_order_destroy(rta_order_model *c)
{
    if (!c) return RTA_ERR_INVALID;
    void *ptrs[] = {c->samples, c->counters, c->params, c->m, c->v, c->grad, c->loss, c->weights, c->partial};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    delete c;
    return RTA_OK;
}

int rta_order_set_params(rta_order_model *c, const float *host_params)
{
    if (!c || !host_params) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaMemcpy(c->params, host_params, kParams * 4, cudaMemcpyHostToDevice));
    k_publish<<<1, 256>>>(c->params, c->weights);
    RTA_CUDA_TRY(cudaGetLastError());
    RTA_CUDA_TRY(cudaDeviceSynchronize());
    return RTA_OK;
}

int rta_order_set_margin(rta_order_model *c, float margin)
{
    if (!c || !(margin >= 0.0f)) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaMemcpy(&c->weights->margin, &margin, 4, cudaMemcpyHostToDevice));
    c->margin = margin;
    return RTA_OK;
}

int rta_order_get_margin(const rta_order_model *c, float *margin)
{
    if (!c || !margin) return RTA_ERR_INVALID;
    *margin = c->margin;
    return RTA_OK;
}

int rta_order_get_params(const rta_order_model *c, float *host_params)
{
    if (!c || !host_params) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaMemcpy(host_params, c->params, kParams * 4, cudaMemcpyDeviceToHost));
    return RTA_OK;
}

int rta_order_clear_samples(rta_order_model *c)
{
    if (!c) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaMemset(c->counters, 0, 4));
    return RTA_OK;
}

int rta_order_sample(rta_order_model *c, const rta_lbvh *bvh, const float *orig, const float *dir,
                     const float *maxt, uint32_t nrays, const uint32_t *d_nrays, void *hits,
                     rta_stream_t stream)
{
    if (!c || !bvh || !orig || !dir || !maxt || !hits || (!d_nrays && nrays == 0) || !c->samples)
        return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    // the ray batches of one call append after the samples already held
    uint32_t before = 0;
    RTA_CUDA_TRY(cudaMemcpy(&before, c->counters, 4, cudaMemcpyDeviceToHost));
    int rc = trace_learn_impl(bvh, nullptr, orig, dir, maxt, nrays, d_nrays, hits, nullptr, c->samples,
                              c->counters, c->cap, c->counters + 1, false, s);
    if (rc) return rc;
    // label this batch's samples from its final hits
    if (before < c->cap)
        k_label<<<1024, 256, 0, s>>>(c->samples, c->counters, c->cap, before, (const HitRec *)hits);
    return check_launch("k_label");
}

int rta_order_sample_count(const rta_order_model *c, uint32_t *n)
{
    if (!c || !n) return RTA_ERR_INVALID;
    uint32_t v = 0;
    RTA_CUDA_TRY(cudaMemcpy(&v, c->counters, 4, cudaMemcpyDeviceToHost));
    *n = v < c->cap ? v : c->cap;
    return RTA_OK;
}

int rta_order_samples(const rta_order_model *c, void **d_samples)
{
    if (!c || !d_samples) return RTA_ERR_INVALID;
    *d_samples = c->samples;
    return RTA_OK;
}

// c->grad += the gradient of `scale` x the loss sum over samples [first,
// first+count), c->loss += that loss sum
static int grad_step(rta_order_model *c, uint32_t first, uint32_t count, float scale, cudaStream_t s)
{
    const uint32_t tiles = (count + 31) / 32;
    uint32_t blocks = (tiles + kGradWarps - 1) / kGradWarps;
    if (blocks > kGradMaxBlocks) blocks = kGradMaxBlocks;
    k_mlp_grad<<<blocks, kGradWarps * 32, sizeof(GradSmem), s>>>(c->weights, c->samples, first, count, scale,
                                                                  c->partial);
    int rc = check_launch("k_mlp_grad");
    if (rc) return rc;
    k_grad_reduce<<<(kParams + 1 + 255) / 256, 256, 0, s>>>(c->partial, blocks, c->grad, c->loss);
    return check_launch("k_grad_reduce");
}

// Gradient of the mean loss over samples [first, first+count) at the current
// parameters, without an update (for checks against a reference).
int rta_order_gradient(rta_order_model *c, uint32_t first, uint32_t count, float *host_grad,
                       float *host_loss)
{
    if (!c || !host_grad || count == 0 || (uint64_t)first + count > c->cap) return RTA_ERR_INVALID;
    RTA_CUDA_TRY(cudaMemset(c->grad, 0, kParams * 4));
    RTA_CUDA_TRY(cudaMemset(c->loss, 0, 4));
    static bool attr = false;
    if (!attr) {
        RTA_CUDA_TRY(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(GradSmem)));
        attr = true;
    }
    int rc = grad_step(c, first, count, 1.0f / (float)count, nullptr);
    if (rc) return rc;
    RTA_CUDA_TRY(cudaMemcpy(host_grad, c->grad, kParams * 4, cudaMemcpyDeviceToHost));
    float l = 0.f;
    RTA_CUDA_TRY(cudaMemcpy(&l, c->loss, 4, cudaMemcpyDeviceToHost));
    if (host_loss) *host_loss = l / (float)count;
    RTA_CUDA_TRY(cudaMemset(c->grad, 0, kParams * 4));
    return RTA_OK;
}

// Adam over the held samples: `epochs` passes of minibatches of `batch` rows.
// The samples are held in the order the traversal recorded them (ray by ray,
// scene by scene), so each epoch visits the minibatches in its own shuffled
// order (Fisher-Yates over the batch indices with the model's hash).
int rta_order_train(rta_order_model *c, uint32_t epochs, uint32_t batch, float lr, float *last_loss,
                    rta_stream_t stream)
{
    if (!c || epochs == 0 || batch == 0) return RTA_ERR_INVALID;
    uint32_t n = 0;
    int rc = rta_order_sample_count(c, &n);
    if (rc) return rc;
    if (n == 0) return RTA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    static bool attr = false;
    if (!attr) {
        RTA_CUDA_TRY(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(GradSmem)));
        attr = true;
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const uint32_t nbatch = (uint32_t)(((uint64_t)n + batch - 1) / batch);
    std::vector<uint32_t> order(nbatch);
    for (uint32_t e = 0; e < epochs; ++e) {
        for (uint32_t i = 0; i < nbatch; ++i) order[i] = i;
        uint32_t h = host_hash(c->seed ^ host_hash((uint32_t)c->step + e));
        for (uint32_t i = nbatch; i > 1; --i) {
            h = host_hash(h + i);
            const uint32_t j = h % i;
            const uint32_t t = order[i - 1];
            order[i - 1] = order[j];
            order[j] = t;
        }
        RTA_CUDA_TRY(cudaMemsetAsync(c->loss, 0, 4, s));
        for (uint32_t bi = 0; bi < nbatch; ++bi) {
            const uint32_t first = order[bi] * batch;
            const uint32_t cnt = n - first < batch ? n - first : batch;
            if ((rc = grad_step(c, first, cnt, 1.0f / (float)cnt, s))) return rc;
            ++c->step;
            const float c1 = 1.f - std::pow(b1, (float)c->step), c2 = 1.f - std::pow(b2, (float)c->step);
            k_adam<<<1, 1024, 0, s>>>(c->params, c->m, c->v, c->grad, lr, b1, b2, c1, c2, eps, c->weights);
            if ((rc = check_launch("rta_order_train"))) return rc;
        }
    }
    if (last_loss) {
        float l = 0.f;
        RTA_CUDA_TRY(cudaStreamSynchronize(s));
        RTA_CUDA_TRY(cudaMemcpy(&l, c->loss, 4, cudaMemcpyDeviceToHost));
        *last_loss = l / (float)n;
    }
    return RTA_OK;
}

int rta_trace_ideal_order(const rta_lbvh *bvh, const float *orig, const float *dir, const float *maxt,
                          uint32_t nrays, const void *known_hits, void *hits, uint32_t *stats,
                          rta_stream_t stream)
{
    if (!bvh || !orig || !dir || !maxt || !known_hits || !hits || nrays == 0) return RTA_ERR_INVALID;
    return trace_learn_impl(bvh, nullptr, orig, dir, maxt, nrays, nullptr, hits, stats, nullptr, nullptr, 0,
                            bvh->status + 4, false, (cudaStream_t)stream, known_hits);
}

int rta_trace_learned(const rta_lbvh *bvh, const rta_order_model *c, const float *orig, const float *dir,
                      const float *maxt, uint32_t nrays, const uint32_t *d_nrays, void *hits,
                      uint32_t *stats, rta_stream_t stream)
{
    if (!bvh || !c || !orig || !dir || !maxt || !hits || (!d_nrays && nrays == 0)) return RTA_ERR_INVALID;
    // A margin no finite logit exceeds: the network never decides, so the
    // order is the plain one and the plain child-is kernel runs it
    if (c->margin >= FLT_MAX)
        return trace_impl(bvh, orig, dir, maxt, nrays, d_nrays, hits, RTA_TRACE_CIS | (stats ? RTA_TRACE_STATS : 0u),
                          stats, c->counters + 1, (cudaStream_t)stream);
    return trace_learn_impl(bvh, c->weights, orig, dir, maxt, nrays, d_nrays, hits, stats, nullptr, nullptr,
                            0, c->counters + 1, true, (cudaStream_t)stream);
}

} // extern "C"
