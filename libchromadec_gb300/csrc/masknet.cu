// masknet.cu -- the learned chroma mask of the Transform-PAL 3D learned form:
// a small 3D convolutional network over one tile's spectrum that predicts,
// for each bin the filter can keep, the fraction of it that is chroma, in
// place of the fixed mirror threshold of TransformPal3D::applyFilter
// (src/decoders/palcolour/transform_pal_3d.cpp:249-333). The reference has no
// learned PAL path; its NTSC nnTransform3D decoder is the precedent for a
// per-bin mask on a 3D tile spectrum (src/decoders/nntransform3d/
// nntransform3d_pipeline_cuda.cu:160-244, 544-567).
//
// Domain of one tile: the 1,280 bins kz 0..7, ky 0..31 (periodic axes of the
// DFT) and q = kx - 2 in 0..4 (zero outside), voxel v = (q * 8 + kz) * 32 + ky.
// Network: input channels f(b) = ln(1 + |X_b|) / 16 and f at b's mirror about
// the carrier, ((10 - kz) mod 8, (40 - ky) mod 32, 4 - q); three 3x3x3
// convolutions of 16 channels with bias and ReLU; a 1x1x1 sigmoid head giving
// p(b). BF16 weights, features and activations, FP32 accumulation. A tile
// whose mean |p - 1/2| is below the confidence limit falls back to the
// threshold decisions.
//
// Kernels:
//  * mn_tc_forward_kernel<TRAIN> (the default forward pass): each
//    convolution as implicit GEMMs on the tensor cores (tcgen05, BF16
//    operands, FP32 accumulators in tensor memory), warp-specialised and
//    persistent over tiles; described where it is defined.
// The CUDA-core kernels (one CTA of 256 threads per tile, persistent over
// tiles; thread t owns the (kz, ky) column t and computes its 5 q x 16
// channels):
//  * mn_forward_kernel<TRAIN>: features -> p (+ fallback flags), the
//    cross-check of the tensor-core pass; the training variant also keeps
//    each layer's activations for the backward pass.
//  * mn_loss_kernel: dL/dz of the head for L = sum |p X - C|^2 / sum |X|^2.
//  * mn_backward_kernel: the head, then per layer the weight gradient (thread
//    (ci, co) sums over the tile's voxels for all 27 taps) and the input
//    gradient (the transposed convolution), each CTA adding into its own
//    slice of a partial-gradient buffer; mn_adam_kernel reduces the slices
//    and takes one Adam step on the FP32 master weights.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/chromadec_gb300.h"
#include "error_state.h"
#include "masknet.h"
#include "tcgen05_ptx.cuh"

namespace chdg {
namespace mn {

constexpr int kThreads = 256;
constexpr int NQ = 5, NZY = 256, NV = 1280, NC = 16, NCIN = 2;
constexpr int CS = 1282;   // channel stride of shared activations (bf16), bank-skewed
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + 27 * NCIN * NC, OFF_W2 = OFF_B1 + NC, OFF_B2 = OFF_W2 + 27 * NC * NC,
              OFF_W3 = OFF_B2 + NC, OFF_B3 = OFF_W3 + 27 * NC * NC, OFF_WH = OFF_B3 + NC, OFF_BH = OFF_WH + NC;
constexpr int NPARAM = OFF_BH + 1;
constexpr int NPARAM_PAD = (NPARAM + 3) & ~3;
static_assert(NPARAM == CHDG_MASKNET_PARAMS, "parameter count");
static_assert(OFF_W2 % 4 == 0 && OFF_W3 % 4 == 0, "float4 weight rows");

__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Accumulate a 3x3x3 convolution of CI input channels into acc[q][co] for
// the thread's column (z, y). in(ci, v) reads input channel ci at voxel v;
// wrow(t, ci) points at the 16 output-channel weights of tap t, input ci
// (stride `wstride` floats between them).
template <int CI, typename In, typename WRow>
__device__ __forceinline__ void conv_acc(const In &in, const WRow &wrow, int z, int y, float (&acc)[NQ][NC])
{
#pragma unroll 1
    for (int dz = -1; dz <= 1; dz++) {
#pragma unroll 1
        for (int dy = -1; dy <= 1; dy++) {
            const int zy = (((z + dz) & 7) << 5) | ((y + dy) & 31);
            const int tb = (dz + 1) * 9 + (dy + 1) * 3;
#pragma unroll 2
            for (int ci = 0; ci < CI; ci++) {
                float xin[NQ + 2];
                xin[0] = 0.f;
                xin[NQ + 1] = 0.f;
#pragma unroll
                for (int q = 0; q < NQ; q++) xin[q + 1] = in(ci, q * NZY + zy);
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    float w[NC];
                    wrow(tb + j, ci, w);
#pragma unroll
                    for (int q = 0; q < NQ; q++) {
                        const float xv = xin[q + j];
#pragma unroll
                        for (int co = 0; co < NC; co++) acc[q][co] = __fmaf_rn(xv, w[co], acc[q][co]);
                    }
                }
            }
        }
    }
}

// Weight rows of a layer's W[27][CI][16] in shared memory (forward)
template <int CI>
struct WFwd {
    const float *W;
    __device__ __forceinline__ void operator()(int t, int ci, float (&w)[NC]) const
    {
        const float4 *p = reinterpret_cast<const float4 *>(W + (t * CI + ci) * NC);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float4 v = p[k];
            w[4 * k] = v.x, w[4 * k + 1] = v.y, w[4 * k + 2] = v.z, w[4 * k + 3] = v.w;
        }
    }
};

// Transposed, flipped rows for the input gradient: input channel = the
// layer's output channel co, outputs = its input channels ci:
// w[ci] = W[26 - t][ci][co]
struct WTrans {
    const float *W;
    __device__ __forceinline__ void operator()(int t, int co, float (&w)[NC]) const
    {
        const float *p = W + (26 - t) * NC * NC + co;
#pragma unroll
        for (int ci = 0; ci < NC; ci++) w[ci] = p[ci * NC];
    }
};

struct InBf16 {
    const __nv_bfloat16 *a;   // [16][CS]
    __device__ __forceinline__ float operator()(int c, int v) const { return __bfloat162float(a[c * CS + v]); }
};

struct InF32 {
    const float *a;   // [CI][NV]
    __device__ __forceinline__ float operator()(int c, int v) const { return a[c * NV + v]; }
};

__device__ __forceinline__ void acc_init(float (&acc)[NQ][NC], const float *bias)
{
#pragma unroll
    for (int q = 0; q < NQ; q++)
#pragma unroll
        for (int co = 0; co < NC; co++) acc[q][co] = bias ? bias[co] : 0.f;
}

// ReLU, round to bf16 and store channel co of the thread's voxels
__device__ __forceinline__ void acc_store_relu(const float (&acc)[NQ][NC], __nv_bfloat16 *out, int zy)
{
#pragma unroll
    for (int q = 0; q < NQ; q++)
#pragma unroll
        for (int co = 0; co < NC; co++) out[co * CS + q * NZY + zy] = __float2bfloat16_rn(fmaxf(acc[q][co], 0.f));
}

// Inputs: the tile's features and their mirror, as two FP32 channels
__device__ __forceinline__ void load_input(const uint16_t *feat_tile, float *x0, int zy)
{
    const int z = zy >> 5, y = zy & 31;
    const int mzy = (((10 - z) & 7) << 5) | ((40 - y) & 31);
    const __nv_bfloat16 *f = reinterpret_cast<const __nv_bfloat16 *>(feat_tile);
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        x0[q * NZY + zy] = __bfloat162float(f[q * NZY + zy]);
        x0[NV + q * NZY + zy] = __bfloat162float(f[(4 - q) * NZY + mzy]);
    }
}

__device__ __forceinline__ void copy_act_out(const __nv_bfloat16 *s, __nv_bfloat16 *g, int zy)
{
    // [16][CS] shared -> [16][NV] global, the thread's column
#pragma unroll
    for (int c = 0; c < NC; c++)
#pragma unroll
        for (int q = 0; q < NQ; q++) g[c * NV + q * NZY + zy] = s[c * CS + q * NZY + zy];
}

__device__ __forceinline__ float block_sum(float v, float *red)
{
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) v += __shfl_xor_sync(0xffffffffu, v, h);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.f;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) s += red[w];
    return s;
}

constexpr size_t kFwdSmem = sizeof(float) * (NPARAM_PAD + 2 * NV) + 2 * sizeof(__nv_bfloat16) * NC * CS;

// params: the network's weights as used (weights bf16-rounded, biases FP32).
// TRAIN: also write A1, A2, A3 ([tile][16][NV] bf16 each) for the backward pass.
template <bool TRAIN>
__global__ void __launch_bounds__(kThreads, 1)
    mn_forward_kernel(const float *params, const uint16_t *feat, long long ntiles, float conf_limit, float *p_out,
                      uint8_t *fallback, __nv_bfloat16 *a1g, __nv_bfloat16 *a2g, __nv_bfloat16 *a3g)
{
    extern __shared__ float4 smem4[];
    float *wsm = reinterpret_cast<float *>(smem4);
    float *x0 = wsm + NPARAM_PAD;
    __nv_bfloat16 *act0 = reinterpret_cast<__nv_bfloat16 *>(x0 + 2 * NV);
    __nv_bfloat16 *act1 = act0 + NC * CS;
    __shared__ float red[kThreads / 32];
    for (int i = threadIdx.x; i < NPARAM; i += kThreads) wsm[i] = params[i];
    const int zy = threadIdx.x, z = zy >> 5, y = zy & 31;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        __syncthreads();   // the previous tile is done with x0 and the activations
        load_input(feat + tile * NV, x0, zy);
        __syncthreads();
        float acc[NQ][NC];
        acc_init(acc, wsm + OFF_B1);
        conv_acc<NCIN>(InF32{x0}, WFwd<NCIN>{wsm + OFF_W1}, z, y, acc);
        acc_store_relu(acc, act0, zy);
        __syncthreads();
        acc_init(acc, wsm + OFF_B2);
        conv_acc<NC>(InBf16{act0}, WFwd<NC>{wsm + OFF_W2}, z, y, acc);
        acc_store_relu(acc, act1, zy);
        __syncthreads();
        acc_init(acc, wsm + OFF_B3);
        conv_acc<NC>(InBf16{act1}, WFwd<NC>{wsm + OFF_W3}, z, y, acc);
        if (TRAIN) {
            copy_act_out(act0, a1g + tile * NC * NV, zy);
            copy_act_out(act1, a2g + tile * NC * NV, zy);
        }
        float conf = 0.f;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            float zh = wsm[OFF_BH];
#pragma unroll
            for (int co = 0; co < NC; co++) {
                const float a = bfr(fmaxf(acc[q][co], 0.f));
                if (TRAIN) a3g[tile * NC * NV + co * NV + q * NZY + zy] = __float2bfloat16_rn(a);
                zh = __fmaf_rn(a, wsm[OFF_WH + co], zh);
            }
            const float p = 1.0f / (1.0f + expf(-zh));
            p_out[tile * NV + q * NZY + zy] = p;
            conf += fabsf(p - 0.5f);
        }
        const float s = block_sum(conf, red);
        if (threadIdx.x == 0 && fallback != nullptr) fallback[tile] = (s * (1.0f / NV) < conf_limit) ? 1 : 0;
    }
}

// sum of a = |X|^2 over the batch (ac: [tile][NV] of (a, c))
__global__ void mn_sum_kernel(const float2 *ac, long long n, double *out)
{
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += (double)ac[i].x;
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) s += __shfl_xor_sync(0xffffffffu, s, h);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// dz = dL/dz_head = 2 (p a - c) / S * p (1 - p); loss partial sums
__global__ void mn_loss_kernel(const float *p, const float2 *ac, long long n, const double *S, float *dz, double *loss)
{
    const float inv = (float)(1.0 / *S);
    double l = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float pv = p[i];
        const float2 v = ac[i];
        const float dp = 2.0f * (pv * v.x - v.y) * inv;
        dz[i] = dp * pv * (1.0f - pv);
        l += (double)((pv * pv * v.x - 2.0f * pv * v.y) * inv);
    }
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) l += __shfl_xor_sync(0xffffffffu, l, h);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// Weight gradient of one layer for the thread's (ci, co):
// g[t] += sum_v in[ci][v + t] * d[co][v]
template <typename In, typename D>
__device__ __forceinline__ void wgrad(const In &in, const D &d, int ci, int co, float (&g)[27])
{
#pragma unroll 1
    for (int zy = 0; zy < NZY; zy++) {
        const int z = zy >> 5, y = zy & 31;
        float dv[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++) dv[q] = d(co, q * NZY + zy);
#pragma unroll
        for (int dz = -1; dz <= 1; dz++) {
#pragma unroll
            for (int dy = -1; dy <= 1; dy++) {
                const int zy2 = (((z + dz) & 7) << 5) | ((y + dy) & 31);
                float xin[NQ + 2];
                xin[0] = 0.f;
                xin[NQ + 1] = 0.f;
#pragma unroll
                for (int q = 0; q < NQ; q++) xin[q + 1] = in(ci, q * NZY + zy2);
                const int tb = (dz + 1) * 9 + (dy + 1) * 3;
#pragma unroll
                for (int j = 0; j < 3; j++)
#pragma unroll
                    for (int q = 0; q < NQ; q++) g[tb + j] = __fmaf_rn(xin[q + j], dv[q], g[tb + j]);
            }
        }
    }
}

constexpr size_t kBwdSmem =
    sizeof(float) * (NPARAM_PAD + 2 * NV + NV) + 2 * sizeof(__nv_bfloat16) * NC * CS;

__device__ __forceinline__ void load_act(const __nv_bfloat16 *g, __nv_bfloat16 *s, int zy)
{
#pragma unroll
    for (int c = 0; c < NC; c++)
#pragma unroll
        for (int q = 0; q < NQ; q++) s[c * CS + q * NZY + zy] = g[c * NV + q * NZY + zy];
}

// The backward pass of the tiles given; each CTA accumulates into
// gpart[blockIdx.x][NPARAM] (zeroed by the caller).
__global__ void __launch_bounds__(kThreads, 1)
    mn_backward_kernel(const float *params, const uint16_t *feat, const __nv_bfloat16 *a1g,
                       const __nv_bfloat16 *a2g, const __nv_bfloat16 *a3g, const float *dzg, long long ntiles,
                       float *gpart)
{
    extern __shared__ float4 smem4[];
    float *wsm = reinterpret_cast<float *>(smem4);
    float *x0 = wsm + NPARAM_PAD;   // [2][NV]
    float *dzs = x0 + 2 * NV;       // [NV]
    __nv_bfloat16 *bufA = reinterpret_cast<__nv_bfloat16 *>(dzs + NV);
    __nv_bfloat16 *bufB = bufA + NC * CS;
    for (int i = threadIdx.x; i < NPARAM; i += kThreads) wsm[i] = params[i];
    const int t = threadIdx.x, zy = t, z = zy >> 5, y = zy & 31;
    const int ci = t >> 4, co = t & 15;   // the thread's weight-gradient pair
    float *gp = gpart + (size_t)blockIdx.x * NPARAM;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        __syncthreads();
        // head: dz, A3
        for (int q = 0; q < NQ; q++) dzs[q * NZY + zy] = dzg[tile * NV + q * NZY + zy];
        load_act(a3g + tile * NC * NV, bufA, zy);
        __syncthreads();
        {
            // d wh[co] = sum_v dz[v] A3[co][v]; d bh = sum_v dz[v] (threads split the voxels)
            const int part = t >> 4;   // 16 parts of 80 voxels
            float s = 0.f, sb = 0.f;
            for (int v = part * 80; v < part * 80 + 80; v++) {
                s = __fmaf_rn(dzs[v], __bfloat162float(bufA[co * CS + v]), s);
                if (co == 0) sb += dzs[v];
            }
            atomicAdd(gp + OFF_WH + co, s);
            if (co == 0) atomicAdd(gp + OFF_BH, sb);
        }
        __syncthreads();
        // dZ3 = bf16(dz * wh[c] * (A3 > 0)), in place
#pragma unroll
        for (int c = 0; c < NC; c++)
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const int e = c * CS + q * NZY + zy;
                const float a = __bfloat162float(bufA[e]);
                bufA[e] = __float2bfloat16_rn(a > 0.f ? dzs[q * NZY + zy] * wsm[OFF_WH + c] : 0.f);
            }
        load_act(a2g + tile * NC * NV, bufB, zy);
        __syncthreads();
        // layer 3: weight and bias gradients, then dA2 -> dZ2 in place of A2
        {
            float g[27];
#pragma unroll
            for (int k = 0; k < 27; k++) g[k] = 0.f;
            wgrad(InBf16{bufB}, InBf16{bufA}, ci, co, g);
#pragma unroll
            for (int k = 0; k < 27; k++) gp[OFF_W3 + (k * NC + ci) * NC + co] += g[k];
            if (ci == 0) {
                float b = 0.f;
                for (int v = 0; v < NV; v++) b += __bfloat162float(bufA[co * CS + v]);
                gp[OFF_B3 + co] += b;
            }
        }
        float acc[NQ][NC];
        acc_init(acc, nullptr);
        conv_acc<NC>(InBf16{bufA}, WTrans{wsm + OFF_W3}, z, y, acc);
        __syncthreads();   // every thread has read A2 for the weight gradient
#pragma unroll
        for (int c = 0; c < NC; c++)
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const int e = c * CS + q * NZY + zy;
                bufB[e] = __float2bfloat16_rn(__bfloat162float(bufB[e]) > 0.f ? acc[q][c] : 0.f);
            }
        load_act(a1g + tile * NC * NV, bufA, zy);   // dZ3 is no longer needed
        __syncthreads();
        // layer 2
        {
            float g[27];
#pragma unroll
            for (int k = 0; k < 27; k++) g[k] = 0.f;
            wgrad(InBf16{bufA}, InBf16{bufB}, ci, co, g);
#pragma unroll
            for (int k = 0; k < 27; k++) gp[OFF_W2 + (k * NC + ci) * NC + co] += g[k];
            if (ci == 0) {
                float b = 0.f;
                for (int v = 0; v < NV; v++) b += __bfloat162float(bufB[co * CS + v]);
                gp[OFF_B2 + co] += b;
            }
        }
        acc_init(acc, nullptr);
        conv_acc<NC>(InBf16{bufB}, WTrans{wsm + OFF_W2}, z, y, acc);
        __syncthreads();
#pragma unroll
        for (int c = 0; c < NC; c++)
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const int e = c * CS + q * NZY + zy;
                bufA[e] = __float2bfloat16_rn(__bfloat162float(bufA[e]) > 0.f ? acc[q][c] : 0.f);
            }
        load_input(feat + tile * NV, x0, zy);
        __syncthreads();
        // layer 1 (two input channels)
        if (ci < NCIN) {
            float g[27];
#pragma unroll
            for (int k = 0; k < 27; k++) g[k] = 0.f;
            wgrad(InF32{x0}, InBf16{bufA}, ci, co, g);
#pragma unroll
            for (int k = 0; k < 27; k++) gp[OFF_W1 + (k * NCIN + ci) * NC + co] += g[k];
        } else if (ci == NCIN) {
            float b = 0.f;
            for (int v = 0; v < NV; v++) b += __bfloat162float(bufA[co * CS + v]);
            gp[OFF_B1 + co] += b;
        }
    }
}

// One Adam step: g = sum over the partial slices (then zeroed); the FP32
// master weights move, and `used` gets the values the kernels compute with
// (weights rounded to bf16, biases as they are).
__global__ void mn_adam_kernel(float *master, float *used, float *m, float *v, float *gpart, int nslices, float lr,
                               float b1, float b2, float eps, float c1, float c2, float *grad_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    float g = 0.f;
    for (int s = 0; s < nslices; s++) {
        g += gpart[(size_t)s * NPARAM + i];
        gpart[(size_t)s * NPARAM + i] = 0.f;
    }
    if (grad_out) grad_out[i] = g;
    if (lr == 0.f) return;
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float w = master[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    master[i] = w;
    const bool bias = (i >= OFF_B1 && i < OFF_W2) || (i >= OFF_B2 && i < OFF_W3) || (i >= OFF_B3 && i < OFF_WH) ||
                      i == OFF_BH;
    used[i] = bias ? w : bfr(w);
}

// Training pairs per bin: (|X|^2, Re(C conj X)) from the composite's and the
// true chroma's spectra
__global__ void mn_pairs_kernel(const float2 *x, const float2 *c, long long n, float2 *ac)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 a = x[i], b = c[i];
        ac[i] = make_float2(a.x * a.x + a.y * a.y, b.x * a.x + b.y * a.y);
    }
}

__global__ void mn_round_kernel(const float *master, float *used)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    const bool bias = (i >= OFF_B1 && i < OFF_W2) || (i >= OFF_B2 && i < OFF_W3) || (i >= OFF_B3 && i < OFF_WH) ||
                      i == OFF_BH;
    used[i] = bias ? master[i] : bfr(master[i]);
}

// ---------------------------------------------------------------------------
// Tensor-core forward pass (tcgen05): each convolution as implicit GEMMs
// ---------------------------------------------------------------------------
// Rows m = ky * 8 + kz (kz fastest: each ky is one 8-row core-matrix group;
// 256 rows, two M blocks of 128), K = (q', ci) of the layer's input, N =
// (q, dz, co): the kz taps are outputs, D_dz(ky, kz) = sum over (dy, q', ci)
// of x(ky + dy - 1, kz) W[dz][dy][q' - q], and the epilogue forms
// y(ky, kz) = sum_dz D_dz(ky, kz + dz - 1) with shuffles inside the 8 lanes
// of each ky (the kz axis is periodic, as the lanes are). A ky tap is an
// offset of whole groups into the one A operand (a periodic halo group on
// both sides). The kx taps fold into N and K: output block q takes input
// block q' through W[.][.][q' - q] for |q' - q| <= 1, so in layers 2 and 3
// the MMAs of one K chunk (input q', its 16 channels) write only the 96 or
// 144 columns of the outputs q = q' - 1 .. q' + 1 (N is ordered q, dz, co).
// Layer 1 (K = 16: the five q' of the two input channels, zero-padded) takes
// the full N = 240. Each M block has its own 240 accumulator columns.
//
// Schedule: the M blocks take turns. A layer's block-0 MMAs, then its block-1
// MMAs, which run while the epilogue empties block 0; block 1's epilogue then
// runs while the next layer's block-0 MMAs go, chunk by chunk as it releases
// them. Block 0's epilogue writes the next layer's input while block 1's MMAs
// still read this layer's: the two row groups both touch (ky = 15, and the
// halo copy of ky = 0) go to a stash that block 1's epilogue moves into place.
//
// Roles (one CTA per SM, persistent over tiles):
//  * warps 0-7, the epilogue, all on one M block at a time: warp w reads
//    tensor-memory lanes 32 (w & 3) .. and the channel half w >> 2 of each
//    output. Per output block q = 0..4 of a layer: read its columns, zero them
//    for the next layer (whose banded MMAs all accumulate), add the dz partial
//    sums, the bias and ReLU, round to bf16 and write K chunk q of the next
//    layer's input; block 1's step q releases the next layer's chunk q. The
//    last layer: the sigmoid head over all 16 channels, warps 0-3 taking
//    output blocks q = 0..2 and warps 4-7 q = 3..4; after block 0's head,
//    warps 4-7 write the next tile's input.
//  * warp 8, one thread: issues the MMAs.
//  * warp 9, one thread: the TMA bulk copies -- the weight pieces of each
//    tile (each used by both M blocks) through a ring of slots, and each next
//    tile's features into one of two stages.
// All waits are bounded; a wait that runs out raises the error flag and the
// CTA leaves after its copies and MMAs in flight have completed.
constexpr int kEpiWarps = 8;
constexpr int kTcThreads = 32 * (kEpiWarps + 2);
constexpr int kGroupsA = 34;                       // 32 ky groups + one halo group on each side
constexpr int A_BYTES = kGroupsA * 8 * 160;        // a layer's input, K up to 80
constexpr int NCOL = 3 * 80;                       // accumulator columns of one M block: (q, dz, co)
constexpr int kSlots = 8;                          // weight-piece ring (a layer's 5 pieces stay for both blocks)
constexpr int SLOT_BYTES = 3 * 144 * 32;           // the largest piece: three ky taps x 144 rows x K 16
constexpr int FEAT_BYTES = NV * 2;
constexpr int kPieces = 10;                        // streamed weight pieces of one tile (layers 2 and 3)
constexpr int W1_BYTES = 3 * NCOL * 32;            // layer 1's weights, resident
constexpr int STASH_BYTES = 2 * 8 * 160;           // row groups 16 and 33 of the next layer's input
constexpr int IN_BYTES = kGroupsA * 8 * 32;        // layer 1's input, K = 16
// shared memory: layers 2 and 3's input [34 groups][8 rows][K 80] and layer
// 1's [34][8][K 16], both canonical (apart, so a tile's input can be written
// while the previous layers' operands are read), the ring, two feature
// stages, the stash, the barriers
constexpr int SM_A = 0;
constexpr int SM_IN = A_BYTES;
constexpr int SM_W1 = SM_IN + IN_BYTES;
constexpr int SM_SLOT = SM_W1 + W1_BYTES;
constexpr int SM_FEAT = SM_SLOT + kSlots * SLOT_BYTES;
constexpr int SM_STASH = SM_FEAT + 2 * FEAT_BYTES;
constexpr int SM_BAR = SM_STASH + STASH_BYTES;
// barriers: an M block's MMAs of a layer done (2); a release of the MMAs (5:
// chunk q of the next layer's input written, and for layer 1 the input (0)
// and block 1's columns read (1)); slot full (kSlots); slot free (kSlots);
// feature stage full (2) and free (2); the final drain of the MMAs; layer
// 1's weights landed
constexpr int B_FULL = 0, B_READY = 2, B_SFULL = B_READY + 5, B_SFREE = B_SFULL + kSlots, B_FFULL = B_SFREE + kSlots,
              B_FFREE = B_FFULL + 2, B_DRAIN = B_FFREE + 2, B_W1 = B_DRAIN + 1, NBAR = B_W1 + 1;
constexpr int SM_TSLOT = SM_BAR + 8 * NBAR;
constexpr int SM_FLAG = SM_TSLOT + 4;
constexpr int kTcSmem = SM_FLAG + 12;
static_assert(kTcSmem + 1024 <= 227 * 1024, "shared memory of one CTA");
static_assert(SM_IN % 16 == 0 && SM_W1 % 16 == 0 && SM_SLOT % 16 == 0 && SLOT_BYTES % 16 == 0 &&
                  SM_FEAT % 16 == 0 && SM_STASH % 16 == 0 && SM_BAR % 8 == 0,
              "copy alignment");

// the band of output blocks of input block (K chunk) ks in layers 2 and 3
__host__ __device__ constexpr int band_lo(int ks) { return ks > 0 ? ks - 1 : 0; }
__host__ __device__ constexpr int band_q(int ks) { return (ks < 4 ? ks + 1 : 4) - band_lo(ks) + 1; }
__host__ __device__ constexpr int band_off(int ks)
{
    int o = 0;
    for (int k = 0; k < ks; k++) o += 3 * 48 * band_q(k) * 32;
    return o;
}
// weight images in global memory, in the order the MMAs take them: layer 1
// [dy][240 rows (q, dz, co)][K 16]; layers 2 and 3 [chunk ks][dy][48 x
// band_q(ks) rows][K 16]; each ky tap's image canonical (8-row groups 256
// bytes apart)
constexpr int IMG_L1 = 0;
constexpr int IMG_L2 = IMG_L1 + 3 * NCOL * 32;
constexpr int IMG_L3 = IMG_L2 + band_off(5);
constexpr int IMG_BYTES = IMG_L3 + band_off(5);
static_assert(band_off(5) == 3 * 48 * 13 * 32, "band sizes");
static_assert(NCOL * 32 <= SLOT_BYTES, "pieces fit a slot");

// Streamed piece p of a tile's weights: source offset and bytes. Pieces
// 0-4: layer 2's chunks; 5-9: layer 3's. Layer 1's weights stay in shared
// memory.
__device__ __forceinline__ void weight_piece(int p, int &off, int &bytes)
{
    const int ks = p % 5;
    off = (p < 5 ? IMG_L2 : IMG_L3) + band_off(ks);
    bytes = 3 * 48 * band_q(ks) * 32;
}

__global__ void mn_build_images_kernel(const float *used, uint8_t *img)
{
    const int n1 = 3 * NCOL * 16, n2 = 3 * 48 * 13 * 16;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n1 + 2 * n2; idx += gridDim.x * blockDim.x) {
        const int k = idx & 15;
        float v = 0.f;
        uint32_t off;
        if (idx < n1) {
            const int n = (idx >> 4) % NCOL, dy = (idx >> 4) / NCOL;
            const int q = n / 48, dz = (n % 48) >> 4, co = n & 15;
            if (k < 5 * NCIN) {
                const int dq = k / NCIN - q, ci = k % NCIN;
                if (dq >= -1 && dq <= 1) v = used[OFF_W1 + (((dz * 3 + dy) * 3 + dq + 1) * NCIN + ci) * NC + co];
            }
            off = IMG_L1 + dy * NCOL * 32 + tpal::tc::elem_off(n, k, 2, 32);
        } else {
            const int r = idx - n1, layer = r < n2 ? 1 : 2, rr = (r % n2) >> 4;
            int ks = 0;
            while (rr >= band_off(ks + 1) / 32) ks++;
            const int nb = 48 * band_q(ks), within = rr - band_off(ks) / 32, dy = within / nb, n = within % nb;
            const int q = band_lo(ks) + n / 48, dz = (n % 48) >> 4, co = n & 15, dq = ks - q;   // |dq| <= 1
            v = used[(layer == 1 ? OFF_W2 : OFF_W3) + (((dz * 3 + dy) * 3 + dq + 1) * NC + k) * NC + co];
            off = (layer == 1 ? IMG_L2 : IMG_L3) + band_off(ks) + dy * nb * 32 + tpal::tc::elem_off(n, k, 2, 32);
        }
        *reinterpret_cast<__nv_bfloat16 *>(img + off) = __float2bfloat16_rn(v);
    }
}

// One 16-byte chunk c of input row (ky, kz) of a layer whose rows hold KB
// bytes: row kz of group ky + 1; groups 0 and 33 repeat ky = 31 and ky = 0
// (the periodic halo).
__device__ __forceinline__ void put_row(uint8_t *A, int KB, int ky, int kz, int c, uint4 v)
{
    const int grp = 8 * KB;
    uint8_t *base = A + c * 128 + kz * 16;
    *reinterpret_cast<uint4 *>(base + (ky + 1) * grp) = v;
    if (ky == 31) *reinterpret_cast<uint4 *>(base) = v;
    if (ky == 0) *reinterpret_cast<uint4 *>(base + (kGroupsA - 1) * grp) = v;
}

// OR of a predicate over the epilogue's 256 threads (named barrier 1).
__device__ __forceinline__ bool epi_or(bool v)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.b32 q, %1, 0;\n\tbar.red.or.pred p, 1, %2, q;\n\t"
                 "selp.b32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(r)
                 : "r"((uint32_t)v), "r"(32 * kEpiWarps)
                 : "memory");
    return r != 0;
}

struct TcShared {
    uint8_t *A, *in, *w1, *slots, *stage;
    uint64_t *bars;
    volatile int *abort_flag;
};

// Descriptor arithmetic: the start address is bits 0-13 of a shared-memory
// descriptor in 16-byte units, so moving an operand by a byte offset that
// keeps it inside shared memory (below 256 KB) adds offset / 16.
__device__ __forceinline__ uint64_t desc_at(uint64_t d, uint32_t bytes) { return d + (bytes >> 4); }

// Layer 1, ky tap DY of one M block from its weight piece: K = 16, N = 240;
// tap 0 starts the block's sum. ab: A at the block's first row group.
template <int DY>
__device__ __forceinline__ void mma_layer1(uint32_t d, uint64_t ab, uint64_t bslot)
{
    tpal::tc::mma<1>(d, desc_at(ab, DY * 256), bslot, tpal::tc::idesc(1, 128, NCOL), DY > 0 ? 1u : 0u);
}

// Layers 2 and 3, K chunk KS (input block q' = KS) of one M block: three ky
// taps into the band's 96 or 144 columns; every MMA accumulates.
template <int KS>
__device__ __forceinline__ void mma_band(uint32_t d, uint64_t ab, uint64_t bslot)
{
    constexpr int nb = 48 * band_q(KS);
    constexpr uint32_t id = tpal::tc::idesc(1, 128, nb);
#pragma unroll
    for (int dy = 0; dy < 3; dy++)
        tpal::tc::mma<1>(d + 48 * band_lo(KS), desc_at(ab, dy * 1280 + KS * 256), desc_at(bslot, dy * nb * 32), id,
                         1u);
}

__device__ __forceinline__ void mma_band_any(int ks, uint32_t d, uint64_t ab, uint64_t bslot)
{
    switch (ks) {
    case 0: mma_band<0>(d, ab, bslot); break;
    case 1: mma_band<1>(d, ab, bslot); break;
    case 2: mma_band<2>(d, ab, bslot); break;
    case 3: mma_band<3>(d, ab, bslot); break;
    default: mma_band<4>(d, ab, bslot); break;
    }
}

// The MMA warp's thread. Per tile and layer: block 0's MMAs (each chunk once
// released), then block 1's with the same weight pieces, whose slots are then
// freed.
__device__ bool tc_mma_role(const TcShared &S, uint32_t tmem, long long first, long long step, long long ntiles)
{
    using namespace tpal::tc;
    uint64_t *full = S.bars + B_FULL, *ready = S.bars + B_READY, *sfull = S.bars + B_SFULL,
             *sfree = S.bars + B_SFREE;
    // operand descriptors at the bases: A with 8-row groups 256 bytes apart
    // (layer 1) or 1280 (layers 2 and 3), the weight slots 256; block 1's A
    // starts 16 row groups in
    const uint64_t a1 = sdesc(smem_addr(S.in), 256), a2 = sdesc(smem_addr(S.A), 1280),
                   b0 = sdesc(smem_addr(S.slots), 256);
    const uint64_t a1b[2] = {a1, desc_at(a1, 16 * 256)}, a2b[2] = {a2, desc_at(a2, 16 * 1280)};
    uint32_t rbits = 0;   // parity of each release barrier's next phase
    long long sc = 0;     // weight pieces taken
    bool ok = true;
    auto take_ready = [&](int q) {
        if (!bar_wait(ready + q, (rbits >> q) & 1)) return false;
        rbits ^= 1u << q;
        fence_after();
        return true;
    };
    // the weight piece p's slot, once its copy has landed
    auto take_slot = [&](long long p) {
        if (!bar_wait(sfull + (int)(p % kSlots), (uint32_t)((p / kSlots) & 1))) return false;
        fence_after();
        return true;
    };
    auto slot_desc = [&](long long p) { return desc_at(b0, (int)(p % kSlots) * SLOT_BYTES); };
    // layer 1's weights, copied once
    const uint64_t w1 = sdesc(smem_addr(S.w1), 256);
    if (ntiles > first) {
        ok = bar_wait(S.bars + B_W1, 0);
        fence_after();
    }
    for (long long tile = first; tile < ntiles && ok && !*S.abort_flag; tile += step) {
        // layer 1: block 0 once the tile's input is written and the previous
        // tile's head has read block 0's columns, block 1 once it has read
        // block 1's
        ok = take_ready(0);
        if (ok) {
            mma_layer1<0>(tmem, a1b[0], w1);
            mma_layer1<1>(tmem, a1b[0], desc_at(w1, NCOL * 32));
            mma_layer1<2>(tmem, a1b[0], desc_at(w1, 2 * NCOL * 32));
        }
        mma_commit(full + 0);
        if (ok) ok = take_ready(1);
        if (ok) {
            mma_layer1<0>(tmem + 256, a1b[1], w1);
            mma_layer1<1>(tmem + 256, a1b[1], desc_at(w1, NCOL * 32));
            mma_layer1<2>(tmem + 256, a1b[1], desc_at(w1, 2 * NCOL * 32));
        }
        mma_commit(full + 1);
        // layers 2 and 3: block 0's chunk ks once block 1's epilogue of the
        // previous layer released it (the weight piece is taken first: it
        // landed long before, so that wait overlaps the epilogue step that
        // releases the chunk); block 1's chunks need nothing more
        for (int L = 1; L < 3 && ok; L++) {
            const long long p = sc;
            for (int ks = 0; ks < 5 && ok; ks++) {
                ok = take_slot(p + ks) && take_ready(ks);
                if (ok) mma_band_any(ks, tmem, a2b[0], slot_desc(p + ks));
            }
            mma_commit(full + 0);
            if (ok) {
                for (int ks = 0; ks < 5; ks++) {
                    mma_band_any(ks, tmem + 256, a2b[1], slot_desc(p + ks));
                    mma_commit(sfree + (int)((p + ks) % kSlots));
                }
            }
            mma_commit(full + 1);
            sc += 5;
        }
    }
    if (!ok) *S.abort_flag = 1;
    // every MMA issued has completed before the tensor memory is released
    mma_commit(S.bars + B_DRAIN);
    return bar_wait(S.bars + B_DRAIN, 0) && ok;
}

// The copy warp's thread: weight pieces through the ring, features of the
// next tile into the other stage.
__device__ bool tc_copy_role(const TcShared &S, const uint8_t *img, const uint16_t *feat, long long first,
                             long long step, long long ntiles)
{
    using namespace tpal::tc;
    uint64_t *sfull = S.bars + B_SFULL, *sfree = S.bars + B_SFREE, *ffull = S.bars + B_FFULL,
             *ffree = S.bars + B_FFREE;
    long long sc = 0;   // pieces issued
    long long js = 0;   // tiles whose features were issued
    bool ok = true;
    auto stage_features = [&](long long tile) {
        const int b = (int)(js & 1);
        const long long use = js >> 1;   // earlier fills of this stage
        if (use >= 1 && !bar_wait(ffree + b, (uint32_t)((use - 1) & 1))) return false;
        bar_arrive_expect_tx(ffull + b, FEAT_BYTES);
        bulk_g2s(S.stage + b * FEAT_BYTES, feat + tile * NV, FEAT_BYTES, ffull + b);
        js++;
        return true;
    };
    if (first < ntiles) {
        bar_arrive_expect_tx(S.bars + B_W1, W1_BYTES);
        bulk_g2s(S.w1, img + IMG_L1, W1_BYTES, S.bars + B_W1);
        ok = stage_features(first);
    }
    for (long long tile = first; tile < ntiles && ok && !*S.abort_flag; tile += step) {
        if (tile + step < ntiles) ok = stage_features(tile + step);
        for (int pc = 0; pc < kPieces && ok; pc++) {
            const int slot = (int)(sc % kSlots);
            const long long use = sc / kSlots;
            if (use >= 1 && !bar_wait(sfree + slot, (uint32_t)((use - 1) & 1))) {
                ok = false;
                break;
            }
            int off, bytes;
            weight_piece(pc, off, bytes);
            bar_arrive_expect_tx(sfull + slot, (uint32_t)bytes);
            bulk_g2s(S.slots + slot * SLOT_BYTES, img + off, (uint32_t)bytes, sfull + slot);
            sc++;
        }
    }
    if (!ok) *S.abort_flag = 1;
    // no copy may still be writing shared memory when the CTA leaves: wait
    // for the last fill of every slot and stage (already complete unless a
    // wait ran out)
    for (int slot = 0; slot < kSlots; slot++)
        if (sc > slot && !bar_wait(sfull + slot, (uint32_t)(((sc - 1 - slot) / kSlots) & 1))) ok = false;
    for (int b = 0; b < 2; b++)
        if (js > b && !bar_wait(ffull + b, (uint32_t)(((js - 1 - b) >> 1) & 1))) ok = false;
    if (first < ntiles && !bar_wait(S.bars + B_W1, 0)) ok = false;
    return ok;
}

// The 24 accumulator columns of output block q and channel half h of the
// thread's lane (q * 48 + dz * 16 + 8 h + c; tl already holds 8 h): loads
// issued, not waited for.
__device__ __forceinline__ void load_half(uint32_t tl, int q, uint32_t (&d)[24])
{
    tpal::tc::tmem_ld8_async(tl + q * 48, &d[0]);
    tpal::tc::tmem_ld8_async(tl + q * 48 + 16, &d[8]);
    tpal::tc::tmem_ld8_async(tl + q * 48 + 32, &d[16]);
}

// The half block's outputs: the three dz partial sums of each channel added
// with the kz neighbours' (lanes of the same ky holding kz - 1 and kz + 1).
__device__ __forceinline__ void combine_half(const uint32_t (&d)[24], int lane, float (&y)[8])
{
    const int lm = (lane & ~7) | ((lane - 1) & 7), lp = (lane & ~7) | ((lane + 1) & 7);
#pragma unroll
    for (int c = 0; c < 8; c++)
        y[c] = __shfl_sync(0xffffffffu, __uint_as_float(d[c]), lm) + __uint_as_float(d[8 + c]) +
               __shfl_sync(0xffffffffu, __uint_as_float(d[16 + c]), lp);
}

// The 48 columns of output block q, all 16 channels (the head).
__device__ __forceinline__ void load_block(uint32_t tl, int q, uint32_t (&d)[48])
{
    uint32_t(&d0)[16] = *reinterpret_cast<uint32_t(*)[16]>(&d[0]);
    uint32_t(&d1)[16] = *reinterpret_cast<uint32_t(*)[16]>(&d[16]);
    uint32_t(&d2)[16] = *reinterpret_cast<uint32_t(*)[16]>(&d[32]);
    tpal::tc::tmem_ld16_async(tl + q * 48, d0);
    tpal::tc::tmem_ld16_async(tl + q * 48 + 16, d1);
    tpal::tc::tmem_ld16_async(tl + q * 48 + 32, d2);
}

__device__ __forceinline__ void combine_block(const uint32_t (&d)[48], int lane, float (&y)[16])
{
    const int lm = (lane & ~7) | ((lane - 1) & 7), lp = (lane & ~7) | ((lane + 1) & 7);
#pragma unroll
    for (int co = 0; co < 16; co++)
        y[co] = __shfl_sync(0xffffffffu, __uint_as_float(d[co]), lm) + __uint_as_float(d[16 + co]) +
                __shfl_sync(0xffffffffu, __uint_as_float(d[32 + co]), lp);
}

template <bool TRAIN>
__global__ void __launch_bounds__(kTcThreads, 1)
    mn_tc_forward_kernel(const uint8_t *img, const float *params, const uint16_t *feat, long long ntiles,
                         float conf_limit, float *p_out, uint8_t *fallback, __nv_bfloat16 *a1g, __nv_bfloat16 *a2g,
                         __nv_bfloat16 *a3g, int *err)
{
    using namespace tpal::tc;
    extern __shared__ __align__(1024) uint8_t smem[];
    TcShared S;
    S.A = smem + SM_A;
    S.in = smem + SM_IN;
    S.w1 = smem + SM_W1;
    S.slots = smem + SM_SLOT;
    S.stage = smem + SM_FEAT;
    S.bars = reinterpret_cast<uint64_t *>(smem + SM_BAR);
    S.abort_flag = reinterpret_cast<volatile int *>(smem + SM_FLAG);
    uint8_t *stash = smem + SM_STASH;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + SM_TSLOT);
    __shared__ float s_par[4 * NC + 1];   // b1, b2, b3, wh, bh
    __shared__ float red[2][kEpiWarps];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int i = t; i < 4 * NC + 1; i += kTcThreads) {
        const int off[5] = {OFF_B1, OFF_B2, OFF_B3, OFF_WH, OFF_BH};
        s_par[i] = params[off[i / NC] + i % NC];
    }
    if (t == 0) {
        for (int i = 0; i < NBAR; i++) {
            const bool per_warp = (i >= B_READY && i < B_READY + 5) || i == B_FFREE || i == B_FFREE + 1;
            bar_init(S.bars + i, per_warp ? kEpiWarps : 1);
        }
        *S.abort_flag = 0;
    }
    if (warp == 0) tmem_alloc(tslot, 512);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    const long long first = blockIdx.x, step = gridDim.x;
    bool ok = true;
    if (warp == kEpiWarps) {
        if (lane == 0) ok = tc_mma_role(S, tmem, first, step, ntiles);
        __syncwarp();
    } else if (warp == kEpiWarps + 1) {
        if (lane == 0) ok = tc_copy_role(S, img, feat, first, step, ntiles);
        __syncwarp();
    } else {
        uint64_t *full = S.bars + B_FULL, *ready = S.bars + B_READY, *ffull = S.bars + B_FFULL,
                 *ffree = S.bars + B_FFREE;
        const int qd = warp & 3, h = warp >> 2;       // lane quadrant, channel half
        const int kz = lane & 7;
        const uint32_t tq = tmem + ((uint32_t)(qd * 32) << 16);   // the warp's lanes, column 0
        uint32_t fbits = 0, pfull = 0;
        long long js = 0;   // tiles whose input was written
        bool bad = false;
        // A tile's input from its feature stage, by warps 4-7 (two rows a
        // thread): row r = (ky, kz), k = 2 q + c (c = 0: the bin, 1: its
        // mirror), zero-padded to 16. Every epilogue warp releases the stage
        // and the first layer's block-0 MMAs.
        auto write_input = [&]() {
            const int b = (int)(js & 1);
            bool done = true;
            if (h == 1) {
                done = bar_wait(ffull + b, (fbits >> b) & 1);
                if (done) {
                    fbits ^= 1u << b;
                    const __nv_bfloat16 *f = reinterpret_cast<const __nv_bfloat16 *>(S.stage + b * FEAT_BYTES);
                    for (int r = t - 128; r < 256; r += 128) {
                        const int ky = r >> 3, rz = r & 7;
                        __align__(16) __nv_bfloat16 v[16];
#pragma unroll
                        for (int q = 0; q < NQ; q++) {
                            v[2 * q] = f[(q * 8 + rz) * 32 + ky];
                            v[2 * q + 1] = f[((4 - q) * 8 + ((10 - rz) & 7)) * 32 + ((40 - ky) & 31)];
                        }
#pragma unroll
                        for (int k = 10; k < 16; k++) v[k] = __float2bfloat16_rn(0.f);
                        put_row(S.in, 32, ky, rz, 0, reinterpret_cast<const uint4 *>(v)[0]);
                        put_row(S.in, 32, ky, rz, 1, reinterpret_cast<const uint4 *>(v)[1]);
                    }
                    fence_async_smem();
                }
            }
            __syncwarp();
            if (lane == 0) {
                bar_arrive(ffree + b);
                bar_arrive(ready + 0);
            }
            js++;
            return done;
        };
        if (first < ntiles) {
            bad = !write_input();
            // block 1's columns are free for the first tile
            if (lane == 0) bar_arrive(ready + 1);
        }
        long long it = 0;
        for (long long tile = first; tile < ntiles; tile += step, it++) {
            float conf = 0.f;
            const bool more = tile + step < ntiles;
            for (int L = 0; L < 3; L++) {
                for (int b = 0; b < 2; b++) {
                    if (bad) break;
                    if (!bar_wait(full + b, (pfull >> b) & 1)) {
                        bad = true;
                        break;
                    }
                    pfull ^= 1u << b;
                    fence_after();
                    const int erow = b * 128 + qd * 32 + lane;   // the row: ky = erow >> 3, kz
                    const int ky = erow >> 3;
                    if (L < 2) {
                        const uint32_t tl = tq + b * 256 + h * 8;
                        float bias[8];
#pragma unroll
                        for (int c = 0; c < 8; c++) bias[c] = s_par[L * NC + h * 8 + c];
                        auto step_q = [&](int q, uint32_t(&cur)[24], uint32_t(&nxt)[24]) {
                            tmem_wait_ld(cur);
                            // cleared for the next layer, whose MMAs all accumulate
                            tmem_zero8(tl + q * 48);
                            tmem_zero8(tl + q * 48 + 16);
                            tmem_zero8(tl + q * 48 + 32);
                            if (q + 1 < NQ) load_half(tl, q + 1, nxt);
                            float y[8];
                            combine_half(cur, lane, y);
                            __align__(16) __nv_bfloat16 o[8];
#pragma unroll
                            for (int c = 0; c < 8; c++)
                                o[c] = __float2bfloat16_rn(fmaxf(y[c] + bias[c], 0.f));
                            const uint4 ov = *reinterpret_cast<const uint4 *>(o);
                            const int ch = 2 * q + h;   // the 16-byte chunk of the input row
                            if (b == 0) {
                                // groups 16 (ky = 15) and 33 (the halo copy of
                                // ky = 0) are still read by block 1's MMAs
                                if (ky == 15)
                                    *reinterpret_cast<uint4 *>(stash + (kz * 10 + ch) * 16) = ov;
                                else
                                    *reinterpret_cast<uint4 *>(S.A + (ky + 1) * 1280 + ch * 128 + kz * 16) = ov;
                                if (ky == 0)
                                    *reinterpret_cast<uint4 *>(stash + ((8 + kz) * 10 + ch) * 16) = ov;
                            } else {
                                put_row(S.A, 160, ky, kz, ch, ov);
                                // the stashed rows of this thread's block-0 twin (same lane)
                                if (ky == 16)
                                    *reinterpret_cast<uint4 *>(S.A + (kGroupsA - 1) * 1280 + ch * 128 + kz * 16) =
                                        *reinterpret_cast<const uint4 *>(stash + ((8 + kz) * 10 + ch) * 16);
                                if (ky == 31)
                                    *reinterpret_cast<uint4 *>(S.A + 16 * 1280 + ch * 128 + kz * 16) =
                                        *reinterpret_cast<const uint4 *>(stash + (kz * 10 + ch) * 16);
                            }
                            if (TRAIN) {
                                __nv_bfloat16 *ag = (L == 0 ? a1g : a2g) + tile * NC * NV;
                                const int vox = (q * 8 + kz) * 32 + ky;
#pragma unroll
                                for (int c = 0; c < 8; c++) ag[(h * 8 + c) * NV + vox] = o[c];
                            }
                            if (b == 1) {
                                // the next layer's input chunk q is complete
                                // (block 0's rows were written before) and
                                // block 1's columns 0..q are read; after the
                                // last step all of them are zeroed
                                fence_async_smem();
                                if (q == NQ - 1) tmem_wait_st();
                                fence_before();
                                __syncwarp();
                                if (lane == 0) bar_arrive(ready + q);
                            }
                        };
                        uint32_t ba[24], bb[24];
                        load_half(tl, 0, ba);
                        step_q(0, ba, bb);
                        step_q(1, bb, ba);
                        step_q(2, ba, bb);
                        step_q(3, bb, ba);
                        step_q(4, ba, bb);
                        if (b == 0) {
                            // block 0's rows and zeroed columns, before block
                            // 1's steps release the next layer's chunks
                            fence_async_smem();
                            tmem_wait_st();
                            fence_before();
                        }
                    } else {
                        // the sigmoid head over the row's 16 channels: warps
                        // 0-3 take output blocks q = 0..2, warps 4-7 q = 3..4
                        const uint32_t tl = tq + b * 256;
                        const float zh0 = s_par[4 * NC];
                        auto head_q = [&](int q, int qend, uint32_t(&cur)[48], uint32_t(&nxt)[48]) {
                            tmem_wait_ld(cur);
                            if (q + 1 < qend) load_block(tl, q + 1, nxt);
                            float y[16];
                            combine_block(cur, lane, y);
                            const int vox = (q * 8 + kz) * 32 + ky;
                            float zh = zh0;
#pragma unroll
                            for (int co = 0; co < NC; co++) {
                                const float a = bfr(fmaxf(y[co] + s_par[2 * NC + co], 0.f));
                                if (TRAIN) a3g[tile * NC * NV + co * NV + vox] = __float2bfloat16_rn(a);
                                zh = __fmaf_rn(a, s_par[3 * NC + co], zh);
                            }
                            const float p = 1.0f / (1.0f + expf(-zh));
                            p_out[tile * NV + vox] = p;
                            conf += fabsf(p - 0.5f);
                        };
                        uint32_t ba[48], bb[48];
                        if (h == 0) {
                            load_block(tl, 0, ba);
                            head_q(0, 3, ba, bb);
                            head_q(1, 3, bb, ba);
                            head_q(2, 3, ba, bb);
                        } else {
                            load_block(tl, 3, ba);
                            head_q(3, 5, ba, bb);
                            head_q(4, 5, bb, ba);
                        }
                        // block b's columns are read: the next tile's layer-1
                        // MMAs of block b may run. During block 0, warps 4-7
                        // then write the next tile's input (layer 1's operand
                        // region is free: this tile's layer-1 MMAs are long
                        // done) and warps 0-3 only release the feature stage.
                        fence_before();
                        __syncwarp();
                        if (more) {
                            if (b == 0) {
                                if (!write_input()) bad = true;
                            } else if (lane == 0) {
                                bar_arrive(ready + 1);
                            }
                        }
                    }
                }
            }
            // the tile's confidence; a failure anywhere stops every epilogue warp here
#pragma unroll
            for (int hh = 16; hh >= 1; hh >>= 1) conf += __shfl_xor_sync(0xffffffffu, conf, hh);
            if (lane == 0) red[it & 1][warp] = conf;
            if (epi_or(bad || *S.abort_flag != 0)) {
                bad = true;
                break;
            }
            if (t == 0 && fallback != nullptr) {
                float sum = 0.f;
#pragma unroll
                for (int w = 0; w < kEpiWarps; w++) sum += red[it & 1][w];
                fallback[tile] = (sum * (1.0f / NV) < conf_limit) ? 1 : 0;
            }
        }
        if (bad) *S.abort_flag = 1;
        ok = !bad;
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
    if (!ok) atomicExch(err, 1);
}

}  // namespace mn

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int mn_fail(const std::string &what, int code = CHDG_E_INVALID_ARG)
{
    chd::detail::set_last_error("chdg_masknet: " + what);
    return code;
}

static int mn_cuda(const char *what, cudaError_t e)
{
    return mn_fail(std::string(what) + ": " + cudaGetErrorString(e), CHDG_E_CUDA);
}

MaskNet::~MaskNet()
{
    for (void *p : {(void *)master_, (void *)used_, (void *)m_, (void *)v_, (void *)gpart_, (void *)a1_, (void *)a2_,
                    (void *)a3_, (void *)p_, (void *)dz_, (void *)scal_, (void *)grad_, (void *)img_, (void *)err_})
        if (p) cudaFree(p);
}

int MaskNet::init()
{
    cudaError_t e;
    const size_t pb = sizeof(float) * mn::NPARAM;
    for (float **p : {&master_, &used_, &m_, &v_, &grad_})
        if ((e = cudaMalloc(p, pb)) != cudaSuccess) return mn_cuda("cudaMalloc", e);
    cudaMemset(m_, 0, pb);
    cudaMemset(v_, 0, pb);
    if ((e = cudaMalloc(&scal_, 2 * sizeof(double))) != cudaSuccess) return mn_cuda("cudaMalloc", e);
    if ((e = cudaMalloc(&img_, mn::IMG_BYTES)) != cudaSuccess) return mn_cuda("cudaMalloc", e);
    if ((e = cudaMalloc(&err_, sizeof(int))) != cudaSuccess) return mn_cuda("cudaMalloc", e);
    cudaMemset(err_, 0, sizeof(int));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_ = sms > 0 ? sms : 1;
    if ((e = cudaMalloc(&gpart_, sizeof(float) * mn::NPARAM * (size_t)grid_)) != cudaSuccess)
        return mn_cuda("cudaMalloc", e);
    cudaMemset(gpart_, 0, sizeof(float) * mn::NPARAM * (size_t)grid_);
    static bool attr[64] = {};
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        const auto a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (cudaFuncSetAttribute(mn::mn_forward_kernel<false>, a, (int)mn::kFwdSmem) != cudaSuccess ||
            cudaFuncSetAttribute(mn::mn_forward_kernel<true>, a, (int)mn::kFwdSmem) != cudaSuccess ||
            cudaFuncSetAttribute(mn::mn_backward_kernel, a, (int)mn::kBwdSmem) != cudaSuccess ||
            cudaFuncSetAttribute(mn::mn_tc_forward_kernel<false>, a, mn::kTcSmem) != cudaSuccess ||
            cudaFuncSetAttribute(mn::mn_tc_forward_kernel<true>, a, mn::kTcSmem) != cudaSuccess)
            return mn_cuda("cudaFuncSetAttribute", cudaGetLastError());
        attr[dev] = true;
    }
    return 0;
}

int MaskNet::set_weights(const float *host, size_t n)
{
    if (n != (size_t)mn::NPARAM) return mn_fail("expected " + std::to_string(mn::NPARAM) + " parameters");
    cudaError_t e = cudaMemcpy(master_, host, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return mn_cuda("cudaMemcpy", e);
    cudaMemset(m_, 0, sizeof(float) * n);
    cudaMemset(v_, 0, sizeof(float) * n);
    step_ = 0;
    mn::mn_round_kernel<<<(mn::NPARAM + 255) / 256, 256>>>(master_, used_);
    if (const int rc = build_images(nullptr); rc != 0) return rc;
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return mn_cuda("round", e);
    return 0;
}

int MaskNet::build_images(cudaStream_t s)
{
    mn::mn_build_images_kernel<<<256, 256, 0, s>>>(used_, img_);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : mn_cuda("weight images", e);
}

int MaskNet::sync(cudaStream_t s) const
{
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mn_cuda("sync", e);
    int h = 0;
    if ((e = cudaMemcpy(&h, err_, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess) return mn_cuda("sync", e);
    if (h != 0) return mn_fail("a tensor-core completion wait ran out", CHDG_E_CUDA);
    return 0;
}

int MaskNet::get_weights(float *host, size_t n) const
{
    if (n != (size_t)mn::NPARAM) return mn_fail("expected " + std::to_string(mn::NPARAM) + " parameters");
    cudaError_t e = cudaMemcpy(host, master_, sizeof(float) * n, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? 0 : mn_cuda("cudaMemcpy", e);
}

int MaskNet::forward(const uint16_t *d_feat, long long ntiles, float *d_p, uint8_t *d_fallback, cudaStream_t s) const
{
    if (ntiles <= 0) return 0;
    if (d_feat == nullptr || d_p == nullptr) return mn_fail("forward: null buffer");
    if (tc_ && reinterpret_cast<uintptr_t>(d_feat) % 16 != 0)
        return mn_fail("forward: the feature buffer must be 16-byte aligned");
    const unsigned blocks = (unsigned)std::min<long long>(ntiles, (long long)grid_ * 1);
    if (tc_)
        mn::mn_tc_forward_kernel<false><<<blocks, mn::kTcThreads, mn::kTcSmem, s>>>(
            img_, used_, d_feat, ntiles, conf_limit_, d_p, d_fallback, nullptr, nullptr, nullptr, err_);
    else
        mn::mn_forward_kernel<false><<<blocks, mn::kThreads, mn::kFwdSmem, s>>>(used_, d_feat, ntiles, conf_limit_,
                                                                                d_p, d_fallback, nullptr, nullptr,
                                                                                nullptr);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : mn_cuda("forward launch", e);
}

int MaskNet::ensure_batch(long long ntiles)
{
    if (ntiles <= cap_) return 0;
    for (void *p : {(void *)a1_, (void *)a2_, (void *)a3_, (void *)p_, (void *)dz_})
        if (p) cudaFree(p);
    a1_ = a2_ = a3_ = nullptr;
    p_ = dz_ = nullptr;
    cap_ = 0;
    cudaError_t e;
    const size_t act = sizeof(uint16_t) * mn::NC * mn::NV * (size_t)ntiles;
    if ((e = cudaMalloc(&a1_, act)) != cudaSuccess || (e = cudaMalloc(&a2_, act)) != cudaSuccess ||
        (e = cudaMalloc(&a3_, act)) != cudaSuccess ||
        (e = cudaMalloc(&p_, sizeof(float) * mn::NV * (size_t)ntiles)) != cudaSuccess ||
        (e = cudaMalloc(&dz_, sizeof(float) * mn::NV * (size_t)ntiles)) != cudaSuccess)
        return mn_cuda("training buffers", e);
    cap_ = ntiles;
    return 0;
}

// Loss and gradients of a batch; with lr > 0 one Adam step follows.
int MaskNet::train_step(const uint16_t *d_feat, const float2 *d_ac, long long ntiles, float lr, double *loss,
                        float *host_grad, cudaStream_t s)
{
    if (ntiles <= 0 || d_feat == nullptr || d_ac == nullptr) return mn_fail("train_step: empty batch or null buffer");
    if (tc_ && reinterpret_cast<uintptr_t>(d_feat) % 16 != 0)
        return mn_fail("train_step: the feature buffer must be 16-byte aligned");
    if (const int rc = ensure_batch(ntiles); rc != 0) return rc;
    const unsigned blocks = (unsigned)std::min<long long>(ntiles, grid_);
    cudaMemsetAsync(scal_, 0, 2 * sizeof(double), s);
    if (tc_)
        mn::mn_tc_forward_kernel<true><<<blocks, mn::kTcThreads, mn::kTcSmem, s>>>(
            img_, used_, d_feat, ntiles, conf_limit_, p_, nullptr, (__nv_bfloat16 *)a1_, (__nv_bfloat16 *)a2_,
            (__nv_bfloat16 *)a3_, err_);
    else
        mn::mn_forward_kernel<true><<<blocks, mn::kThreads, mn::kFwdSmem, s>>>(
            used_, d_feat, ntiles, conf_limit_, p_, nullptr, (__nv_bfloat16 *)a1_, (__nv_bfloat16 *)a2_,
            (__nv_bfloat16 *)a3_);
    const long long n = ntiles * mn::NV;
    mn::mn_sum_kernel<<<256, 256, 0, s>>>(d_ac, n, scal_);
    mn::mn_loss_kernel<<<256, 256, 0, s>>>(p_, d_ac, n, scal_, dz_, scal_ + 1);
    mn::mn_backward_kernel<<<blocks, mn::kThreads, mn::kBwdSmem, s>>>(
        used_, d_feat, (const __nv_bfloat16 *)a1_, (const __nv_bfloat16 *)a2_, (const __nv_bfloat16 *)a3_, dz_,
        ntiles, gpart_);
    float c1 = 1.f, c2 = 1.f;
    if (lr > 0.f) {
        step_++;
        c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)step_)));
        c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)step_)));
    }
    mn::mn_adam_kernel<<<(mn::NPARAM + 255) / 256, 256, 0, s>>>(master_, used_, m_, v_, gpart_, (int)blocks, lr, 0.9f,
                                                               0.999f, 1e-8f, c1, c2, grad_);
    if (lr > 0.f)
        if (const int rc = build_images(s); rc != 0) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mn_cuda("train launch", e);
    if (loss != nullptr || host_grad != nullptr) {
        if (const int rc = sync(s); rc != 0) return rc;
        if (loss != nullptr) {
            double h[2];
            cudaMemcpy(h, scal_, sizeof(h), cudaMemcpyDeviceToHost);
            *loss = h[1];
        }
        if (host_grad != nullptr)
            if ((e = cudaMemcpy(host_grad, grad_, sizeof(float) * mn::NPARAM, cudaMemcpyDeviceToHost)) != cudaSuccess)
                return mn_cuda("gradient copy", e);
    }
    return 0;
}

}  // namespace chdg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct chdg_masknet {
    chdg::MaskNet net;
};

namespace chdg {
MaskNet *masknet_of(chdg_masknet *n) { return &n->net; }
}  // namespace chdg

#pragma GCC visibility push(default)
extern "C" {
int chdg_masknet_create(chdg_masknet **out)
{
    if (out == nullptr) return chdg::mn_fail("create: null argument");
    *out = nullptr;
    auto n = new (std::nothrow) chdg_masknet;
    if (n == nullptr) return chdg::mn_fail("create: out of memory", CHDG_E_OOM);
    if (const int rc = n->net.init(); rc != 0) {
        delete n;
        return rc;
    }
    *out = n;
    return 0;
}

void chdg_masknet_free(chdg_masknet *n) { delete n; }

int chdg_masknet_set_weights(chdg_masknet *n, const float *w, int64_t count)
{
    if (n == nullptr || w == nullptr) return chdg::mn_fail("set_weights: null argument");
    return n->net.set_weights(w, (size_t)count);
}

int chdg_masknet_get_weights(const chdg_masknet *n, float *w, int64_t count)
{
    if (n == nullptr || w == nullptr) return chdg::mn_fail("get_weights: null argument");
    return n->net.get_weights(w, (size_t)count);
}

int chdg_masknet_set_confidence(chdg_masknet *n, float limit)
{
    if (n == nullptr || !(limit >= 0.f && limit <= 0.5f)) return chdg::mn_fail("set_confidence: limit must be in [0, 0.5]");
    n->net.set_confidence(limit);
    return 0;
}

int chdg_masknet_set_tensor_cores(chdg_masknet *n, int32_t on)
{
    if (n == nullptr) return chdg::mn_fail("set_tensor_cores: null network");
    n->net.set_tensor_cores(on != 0);
    return 0;
}

int chdg_masknet_sync(const chdg_masknet *n, void *stream)
{
    if (n == nullptr) return chdg::mn_fail("sync: null network");
    return n->net.sync((cudaStream_t)stream);
}

int chdg_masknet_forward(const chdg_masknet *n, const uint16_t *d_feat, int64_t ntiles, float *d_p,
                         uint8_t *d_fallback, void *stream)
{
    if (n == nullptr) return chdg::mn_fail("forward: null network");
    return n->net.forward(d_feat, ntiles, d_p, d_fallback, (cudaStream_t)stream);
}

int chdg_masknet_train_step(chdg_masknet *n, const uint16_t *d_feat, const float *d_ac, int64_t ntiles,
                            float learning_rate, double *loss, float *grad, void *stream)
{
    if (n == nullptr) return chdg::mn_fail("train_step: null network");
    if (!(learning_rate >= 0.f)) return chdg::mn_fail("train_step: learning rate must be >= 0");
    return n->net.train_step(d_feat, reinterpret_cast<const float2 *>(d_ac), ntiles, learning_rate, loss, grad,
                             (cudaStream_t)stream);
}

int chdg_masknet_pairs(const float *d_spec_x, const float *d_spec_c, int64_t nbins, float *d_ac, void *stream)
{
    if (d_spec_x == nullptr || d_spec_c == nullptr || d_ac == nullptr || nbins < 0)
        return chdg::mn_fail("pairs: bad arguments");
    if (nbins == 0) return 0;
    chdg::mn::mn_pairs_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(d_spec_x),
                                                                       reinterpret_cast<const float2 *>(d_spec_c),
                                                                       nbins, reinterpret_cast<float2 *>(d_ac));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : chdg::mn_cuda("pairs launch", e);
}

}  // extern "C"
#pragma GCC visibility pop
