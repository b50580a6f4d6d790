// tc3d.cu -- tensor-core form of the Transform-PAL 3D forward transform on
// sm_103a: the DFT stages of every tile as matrix contractions on the
// 5th-generation tensor cores (tcgen05.mma, accumulators in tensor memory),
// with split-precision products. A precision study beside the plain form
// (tpal3d.cu), which stays the decoder: it answers how far tensor-core
// spectra move from the FP64 ones and how many threshold decisions that
// flips.
//
// The spectra are the reference's (TransformPal3D::forwardFFTTile,
// src/decoders/palcolour/transform_pal_3d.cpp:168-202): 8 fields x 32 frame
// lines x 16 samples, raised-cosine windowed in all three axes, rows of the
// other field parity and outside the active lines black, bins kx = 2..6 --
// the ones the filter reads (transform_pal_3d.cpp:294-331). Black is
// subtracted first (the raised cosine's spectrum lives on kx in {0, +-1}, so
// kx >= 2 is unchanged), leaving integer samples below 2^17 in magnitude.
//
// The separable DFT runs in three contractions, each a real GEMM with the
// window folded into its coefficient matrix B (K-major, N x K):
//
//   X   rows (tile, row i) x 16 samples        . B_X [10 (5 kx re/im) x 16]
//   Y   rows (tile, kx) x [re(16 rows) | im]   . B_Y [64 (32 ky re/im) x 32]  (per row parity y0)
//   Z   rows (tile, kx, ky) x [re(8 z) | im]   . B_Z [16 (8 kz re/im) x 16]
//
// Split products: an operand a becomes a_hi + a_lo in the MMA's input type
// (TF32: 10 stored mantissa bits, BF16: 7) and each contraction is three MMAs
// accumulating in FP32 in tensor memory, small terms first:
// a_lo.b_hi + a_hi.b_lo + a_hi.b_hi. Variant 0 is 3xTF32 (kind::tf32),
// variant 1 is BF16x3 (kind::f16 with BF16 inputs).
//
// Kernels (one CTA of 128 threads; thread t owns tensor-memory lane t):
//  * tc3_xy_kernel: a unit is 24 spatial tiles of one field. The X stage is
//    three M = 128 MMAs (384 rows = 24 tiles x 16 own-parity rows); its
//    results are read back with tcgen05.ld, split, and written as the Y
//    stage's A operand (120 rows = 24 tiles x 5 kx); one M = 128, N = 64 MMA
//    chain gives S_f[tile][kx][ky].
//  * tc3_z_kernel: 128 rows (Z tile, spatial tile, kx, ky) per block, each
//    gathering the 8 fields' S_f; one N = 16 MMA chain gives S[kz][kx][ky].
// Shared-memory operands use the no-swizzle K-major canonical layout: 8-row x
// 16-byte core matrices, K-adjacent core matrices 128 B apart (leading byte
// offset), 8-row groups a whole row-group apart (stride byte offset). Every
// wait on an MMA completion has an iteration limit; running out sets an error
// flag that chdg_tc3d_sync reports, and the CTA frees its tensor memory and
// returns.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/chromadec_gb300.h"
#include "error_state.h"
#include "tcgen05_ptx.cuh"
#include "tpal_kernels.h"

namespace tpal {
namespace tc {

constexpr int kThreads = 128;
constexpr int kTilesPerUnit = 24;      // X rows 384 = 3 MMAs of 128; Y rows 120
constexpr int kXRows = kTilesPerUnit * 16;
constexpr int kYRows = kTilesPerUnit * 5;
constexpr int kQ = 160;                // (kx, ky) per spatial tile: 5 x 32
constexpr int kSpecPerTile = 8 * kQ;   // (kz, kx, ky)

struct Params {
    const uint16_t *fields;              // buffer holding fields [field_base, ...)
    const uint16_t *const *field_ptrs;   // unused (null): the tensor-core form reads one buffer
    long long field_stride;
    int field_base;
    int nfields, fw, fh, fafl, lafl, black, swap;
    int tileX0, tileY0, ntx, nty, ntiles;
    int f_begin, nf;           // XY stage: fields [f_begin, f_begin + nf)
    int nm;                    // Z stage: Z tiles m_begin .. m_begin + nm - 1 (fields 2m .. 2m+7)
    const uint8_t *bx, *by, *bz;   // forward operand images: [split][...], by [y0][split][...]
    const uint8_t *bzi, *byi, *bxi;   // inverse operand images: bzi [split], byi [y0][split], bxi [split]
    float2 *sf;                // XY output: [nf][ntiles][kQ] (kx major, ky minor)
    float2 *spec;              // Z output: [nm][ntiles][8 kz][kQ]
    // decode (Z forward + decisions + Z inverse, then Y/X inverse and overlap-add)
    float t2f;                 // squared threshold
    float2 *rz;                // [nm][ntiles][4 slices z = 0, 1, 4, 5][kQ]
    int frame0, nout;          // output fields 2 frame0 .. 2 frame0 + nout - 1
    float *partial;            // overlap-class planes, output field (out_field0 + o)
    long long part_class_stride, part_field_stride;
    int part_row_stride, fl_lo, avs, ave, out_field0;
    int *err;
};

template <int KIND>
struct Split;

// put: one element; put_chunk: the ce elements of one 16-byte core-matrix
// row (offset 16-byte aligned) with one vector store per split.
template <>
struct Split<0> {   // TF32: hi = a rounded to 10 stored mantissa bits (to nearest, ties away), lo = the rest rounded
    static constexpr int eb = 4, ce = 4;
    __device__ __forceinline__ static void split(float a, uint32_t &h, uint32_t &l)
    {
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(a));
        h &= 0xFFFFE000u;
        const float rest = a - __uint_as_float(h);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(rest));
        l &= 0xFFFFE000u;
    }
    __device__ __forceinline__ static void put(uint8_t *hi, uint8_t *lo, uint32_t off, float a)
    {
        uint32_t h, l;
        split(a, h, l);
        *reinterpret_cast<uint32_t *>(hi + off) = h;
        *reinterpret_cast<uint32_t *>(lo + off) = l;
    }
    __device__ __forceinline__ static void put_chunk(uint8_t *hi, uint8_t *lo, uint32_t off, const float *v)
    {
        uint32_t h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; j++) split(v[j], h[j], l[j]);
        *reinterpret_cast<uint4 *>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
};

template <>
struct Split<1> {   // BF16: hi = bf16(a), lo = bf16(a - hi), both round to nearest even
    static constexpr int eb = 2, ce = 8;
    __device__ __forceinline__ static void put(uint8_t *hi, uint8_t *lo, uint32_t off, float a)
    {
        const __nv_bfloat16 h = __float2bfloat16_rn(a);
        const __nv_bfloat16 l = __float2bfloat16_rn(a - __bfloat162float(h));
        *reinterpret_cast<__nv_bfloat16 *>(hi + off) = h;
        *reinterpret_cast<__nv_bfloat16 *>(lo + off) = l;
    }
    __device__ __forceinline__ static void put_chunk(uint8_t *hi, uint8_t *lo, uint32_t off, const float *v)
    {
        uint32_t h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const __nv_bfloat162 hh = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
            const float2 hf = __bfloat1622float2(hh);
            const __nv_bfloat162 ll = __floats2bfloat162_rn(v[2 * j] - hf.x, v[2 * j + 1] - hf.y);
            h[j] = *reinterpret_cast<const uint32_t *>(&hh);
            l[j] = *reinterpret_cast<const uint32_t *>(&ll);
        }
        *reinterpret_cast<uint4 *>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
};

// All N elements of row r (N a multiple of the chunk) with vector stores.
template <int KIND, int N>
__device__ __forceinline__ void put_row(uint8_t *hi, uint8_t *lo, int r, int row_bytes, const float (&v)[N])
{
    using SP = Split<KIND>;
#pragma unroll
    for (int c = 0; c < N / SP::ce; c++)
        SP::put_chunk(hi, lo, elem_off(r, c * SP::ce, SP::eb, row_bytes), v + c * SP::ce);
}

// Shared-memory plan of the XY kernel (bytes), every region 1024-aligned.
template <int KIND>
struct XYLayout {
    static constexpr int eb = Split<KIND>::eb;
    static constexpr int rbx = 16 * eb;   // X rows: 16 samples
    static constexpr int rby = 32 * eb;   // Y rows: 16 re + 16 im
    static constexpr int ax_blk = 128 * rbx;
    static constexpr int ax = 0;                              // [split][3 blocks][128 rows]
    // the Y operand reuses the X operand's space: it is written once the X
    // MMAs are complete, and the next X operand once the Y MMAs are
    static constexpr int ay = ax;                             // [split][128 rows]
    static_assert(2 * 128 * rby <= 2 * 3 * ax_blk, "Y operand fits the X operand's space");
    static constexpr int bx = ax + 2 * 3 * ax_blk;            // [split][16 rows]
    static constexpr int by = bx + ((2 * 16 * rbx + 1023) & ~1023);   // [y0][split][64 rows]
    static constexpr int bar = by + 2 * 2 * 64 * rby;
    static constexpr int bytes = bar + 64;
    static constexpr int ksx = rbx / 32;   // MMA K steps (32 bytes each)
    static constexpr int ksy = rby / 32;
};

template <int KIND>
struct ZLayout {
    static constexpr int eb = Split<KIND>::eb;
    static constexpr int rbz = 16 * eb;
    static constexpr int az = 0;                   // [split][128 rows]
    static constexpr int bz = az + 2 * 128 * rbz;  // [split][16 rows]
    static constexpr int bar = bz + ((2 * 16 * rbz + 1023) & ~1023);
    static constexpr int bytes = bar + 64;
    static constexpr int ksz = rbz / 32;
};

__device__ __forceinline__ void copy_image(uint8_t *dst, const uint8_t *src, int bytes)
{
    for (int o = threadIdx.x * 16; o < bytes; o += kThreads * 16)
        *reinterpret_cast<uint4 *>(dst + o) = __ldg(reinterpret_cast<const uint4 *>(src + o));
}

// the three split products into one accumulator: lo.hi, hi.lo, hi.hi
template <int KIND>
__device__ __forceinline__ void mma3(uint32_t dtmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi, uint32_t b_lo,
                                     uint32_t a_sbo, uint32_t b_sbo, int ksteps, uint32_t id)
{
    for (int s = 0; s < ksteps; s++) {
        const uint32_t o = 256u * s;   // two K-adjacent core matrices per step
        mma<KIND>(dtmem, sdesc(a_lo + o, a_sbo), sdesc(b_hi + o, b_sbo), id, s > 0 ? 1u : 0u);
        mma<KIND>(dtmem, sdesc(a_hi + o, a_sbo), sdesc(b_lo + o, b_sbo), id, 1u);
        mma<KIND>(dtmem, sdesc(a_hi + o, a_sbo), sdesc(b_hi + o, b_sbo), id, 1u);
    }
}

// ---------------------------------------------------------------------------
// X and Y stages: S_f[tile][kx][ky] of fields [f_begin, f_begin + nf)
// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(kThreads) tc3_xy_kernel(Params P)
{
    using LY = XYLayout<KIND>;
    using SP = Split<KIND>;
    constexpr int eb = LY::eb;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + LY::bar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + LY::bar + 8);
    const int t = threadIdx.x, warp = t >> 5;

    // coefficient images (both row parities); the Y operand's rows 120..127
    // hold X-operand data, and their outputs are never stored
    copy_image(smem + LY::bx, P.bx, 2 * 16 * LY::rbx);
    copy_image(smem + LY::by, P.by, 2 * 2 * 64 * LY::rby);
    if (t == 0) bar_init(bar);
    if (warp == 0) tmem_alloc(tslot, 128);   // X accumulators: columns 0..47; Y: 64..127
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    uint32_t phase = 0;

    uint8_t *ax_hi = smem + LY::ax, *ax_lo = smem + LY::ax + 3 * LY::ax_blk;
    uint8_t *ay_hi = smem + LY::ay, *ay_lo = smem + LY::ay + 128 * LY::rby;
    const int groups = (P.ntiles + kTilesPerUnit - 1) / kTilesPerUnit;
    const int units = P.nf * groups;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const int fi = u / groups;
        const int tile0 = (u % groups) * kTilesPerUnit;
        const int f = P.f_begin + fi;
        const bool fvalid = f >= 0 && f < P.nfields;
        const int p = (f & 1) ^ P.swap;
        const uint16_t *fp = fvalid ? P.fields + (long long)(f - P.field_base) * P.field_stride : nullptr;

        // 1. X operand: rows (tile, i), samples minus black
        for (int R = t; R < kXRows; R += kThreads) {
            const int ft = R >> 4, i = R & 15;
            const int tile = tile0 + ft;
            float a[16];
#pragma unroll
            for (int x = 0; x < 16; x++) a[x] = 0.f;
            if (fvalid && tile < P.ntiles) {
                const int tileX = P.tileX0 + 8 * (tile % P.ntx);
                const int tileY = P.tileY0 + 16 * (tile / P.ntx);
                const int y0 = (p - tileY) & 1;
                const int L = tileY + y0 + 2 * i;
                if (L >= P.fafl && L <= P.lafl) {
                    const long long last = (long long)P.fh * P.fw - 1;
                    const long long first = (long long)(L >> 1) * P.fw + tileX;   // flat, as the reference reads
                    if (first >= 1 && first + 18 <= last) {
                        // nine aligned 32-bit words lined up by a funnel shift
                        // (rows start on any 2-byte boundary)
                        const uintptr_t pa = reinterpret_cast<uintptr_t>(fp + first);
                        const uint32_t *w = reinterpret_cast<const uint32_t *>(pa & ~(uintptr_t)3);
                        const unsigned sh = (unsigned)(pa & 2) * 8u;
                        uint32_t wd[9];
#pragma unroll
                        for (int k = 0; k < 9; k++) wd[k] = __ldg(w + k);
#pragma unroll
                        for (int k = 0; k < 8; k++) {
                            const uint32_t v = __funnelshift_r(wd[k], wd[k + 1], sh);
                            a[2 * k] = (float)((int)(v & 0xFFFFu) - P.black);
                            a[2 * k + 1] = (float)((int)(v >> 16) - P.black);
                        }
                    } else {
#pragma unroll
                        for (int x = 0; x < 16; x++) {
                            long long idx = first + x;
                            idx = idx < 0 ? 0 : (idx > last ? last : idx);
                            a[x] = (float)((int)__ldg(fp + idx) - P.black);
                        }
                    }
                }
            }
            const int blk = R >> 7, r = R & 127;
            put_row<KIND, 16>(ax_hi + blk * LY::ax_blk, ax_lo + blk * LY::ax_blk, r, LY::rbx, a);
        }
        fence_async_smem();
        __syncthreads();

        // 2. X MMAs: block b -> tensor columns 16 b
        if (t == 0) {
            fence_after();
            for (int b = 0; b < 3; b++)
                mma3<KIND>(tmem + 16 * b, smem_addr(ax_hi + b * LY::ax_blk), smem_addr(ax_lo + b * LY::ax_blk),
                           smem_addr(smem + LY::bx), smem_addr(smem + LY::bx + 16 * LY::rbx), 8 * LY::rbx,
                           8 * LY::rbx, LY::ksx, idesc(KIND == 0 ? 2 : 1, 128, 16));
            mma_commit(bar);
        }
        bool ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();

        // 3. X results -> Y operand rows (tile, kx), columns [re(i) | im(i)]
        for (int b = 0; b < 3; b++) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + 16 * b, v);
            const int R = 128 * b + t;
            const int ft = R >> 4, i = R & 15;
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const int ry = ft * 5 + k;
                SP::put(ay_hi, ay_lo, elem_off(ry, i, eb, LY::rby), v[2 * k]);
                SP::put(ay_hi, ay_lo, elem_off(ry, 16 + i, eb, LY::rby), v[2 * k + 1]);
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();

        // 4. Y MMAs with the coefficients of this field's row parity
        if (t == 0) {
            fence_after();
            // tileY0 + 16 ty keeps the parity of tileY0 for every tile
            const int y0 = (p - P.tileY0) & 1;
            const uint8_t *byh = smem + LY::by + (2 * y0) * 64 * LY::rby;
            mma3<KIND>(tmem + 64, smem_addr(ay_hi), smem_addr(ay_lo), smem_addr(byh), smem_addr(byh + 64 * LY::rby),
                       8 * LY::rby, 8 * LY::rby, LY::ksy, idesc(KIND == 0 ? 2 : 1, 128, 64));
            mma_commit(bar);
        }
        ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();

        // 5. row t = (tile, kx): 32 complex ky, stored contiguously
        {
            const int ft = t / 5, k = t % 5;
            const int tile = tile0 + ft;
            float2 *dst = P.sf + ((long long)fi * P.ntiles + tile) * kQ + k * 32;
            for (int c = 0; c < 4; c++) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + 64 + 16 * c, v);
                if (t < kYRows && tile < P.ntiles) {   // rows start on 256-byte boundaries: pairs of bins per store
                    float4 *d4 = reinterpret_cast<float4 *>(dst + 8 * c);
#pragma unroll
                    for (int j = 0; j < 4; j++) d4[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                }
            }
        }
        fence_before();
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
// Z stage: S[m][tile][kz][kx][ky] from the 8 fields 2m .. 2m+7
// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(kThreads) tc3_z_kernel(Params P)
{
    using LY = ZLayout<KIND>;
    using SP = Split<KIND>;
    constexpr int eb = LY::eb;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + LY::bar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + LY::bar + 8);
    const int t = threadIdx.x, warp = t >> 5;

    copy_image(smem + LY::bz, P.bz, 2 * 16 * LY::rbz);
    if (t == 0) bar_init(bar);
    if (warp == 0) tmem_alloc(tslot, 32);
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    uint32_t phase = 0;
    uint8_t *az_hi = smem + LY::az, *az_lo = smem + LY::az + 128 * LY::rbz;

    const long long rows = (long long)P.nm * P.ntiles * kQ;
    const long long nblk = (rows + 127) / 128;
    for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const long long g = blk * 128 + t;
        const bool valid = g < rows;
        int mi = 0, tile = 0, q = 0;
        float re[8], im[8];
#pragma unroll
        for (int z = 0; z < 8; z++) re[z] = im[z] = 0.f;
        if (valid) {
            mi = (int)(g / ((long long)P.ntiles * kQ));
            const long long rem = g % ((long long)P.ntiles * kQ);
            tile = (int)(rem / kQ);
            q = (int)(rem % kQ);
#pragma unroll
            for (int z = 0; z < 8; z++) {
                const float2 s = P.sf[((long long)(2 * mi + z) * P.ntiles + tile) * kQ + q];
                re[z] = s.x;
                im[z] = s.y;
            }
        }
#pragma unroll
        for (int z = 0; z < 8; z++) {
            SP::put(az_hi, az_lo, elem_off(t, z, eb, LY::rbz), re[z]);
            SP::put(az_hi, az_lo, elem_off(t, 8 + z, eb, LY::rbz), im[z]);
        }
        fence_async_smem();
        __syncthreads();
        if (t == 0) {
            fence_after();
            mma3<KIND>(tmem, smem_addr(az_hi), smem_addr(az_lo), smem_addr(smem + LY::bz),
                       smem_addr(smem + LY::bz + 16 * LY::rbz), 8 * LY::rbz, 8 * LY::rbz, LY::ksz,
                       idesc(KIND == 0 ? 2 : 1, 128, 16));
            mma_commit(bar);
        }
        const bool ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16), v);
        if (valid) {
            float2 *dst = P.spec + ((long long)mi * P.ntiles + tile) * kSpecPerTile + q;
#pragma unroll
            for (int kz = 0; kz < 8; kz++) dst[kz * kQ] = make_float2(v[2 * kz], v[2 * kz + 1]);
        }
        fence_before();
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// Decode: Z forward, threshold decisions and Z inverse of one Z tile of one
// spatial tile per CTA iteration (160 rows (kx, ky) as two M = 128 blocks).
// The decision is the plain form's FP32 rule on the tensor-core spectrum:
// keep a bin when |bin|^2 and |mirror|^2 are within t^2 of each other, the
// mirror about the carrier being ((10 - kz) & 7, 8 - kx, (40 - ky) & 31)
// (transform_pal_3d.cpp:294-331; the carrier, its own mirror, is kept). The
// inverse Z DFT is evaluated only at the four slices an output field takes:
// z = 0, 1 (fields 2m, 2m+1) and z = 4, 5 (fields 2m+4, 2m+5,
// transform_pal_3d.cpp:214-215).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool keep_pair(float a, float b, float t2)
{
    return (__fmaf_rn(-b, t2, a) >= 0.f) && (__fmaf_rn(-a, t2, b) >= 0.f);
}

template <int KIND>
struct ZDLayout {
    static constexpr int eb = Split<KIND>::eb;
    static constexpr int rb = 16 * eb;
    static constexpr int blk = 128 * rb;
    static constexpr int af = 0;                     // [split][2 blocks][128 rows]
    // the inverse operand reuses the forward one's space (written once the
    // forward MMAs are complete; rows 160..255 stay zero in both)
    static constexpr int ai = af;
    static constexpr int bf = af + 4 * blk;          // [split][16 rows]
    static constexpr int bi = bf + 2 * 16 * rb;      // [split][16 rows]
    static constexpr int mag = bi + 2 * 16 * rb;     // [160][8] floats
    static constexpr int bar = mag + kQ * 8 * 4;
    static constexpr int bytes = bar + 64;
    static constexpr int ks = rb / 32;
};

template <int KIND>
__global__ void __launch_bounds__(kThreads) tc3_zd_kernel(Params P)
{
    using LY = ZDLayout<KIND>;
    using SP = Split<KIND>;
    constexpr int eb = LY::eb;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + LY::bar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + LY::bar + 8);
    float *mag = reinterpret_cast<float *>(smem + LY::mag);
    const int t = threadIdx.x, warp = t >> 5;

    copy_image(smem + LY::bf, P.bz, 2 * 16 * LY::rb);
    copy_image(smem + LY::bi, P.bzi, 2 * 16 * LY::rb);
    for (int o = t * 16; o < 4 * LY::blk; o += kThreads * 16) *reinterpret_cast<uint4 *>(smem + LY::af + o) = uint4{0, 0, 0, 0};
    if (t == 0) bar_init(bar);
    if (warp == 0) tmem_alloc(tslot, 64);   // forward: columns 0..31, inverse: 32..63
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    uint32_t phase = 0;
    uint8_t *af_hi = smem + LY::af, *af_lo = smem + LY::af + 2 * LY::blk;
    uint8_t *ai_hi = smem + LY::ai, *ai_lo = smem + LY::ai + 2 * LY::blk;
    const uint32_t id = idesc(KIND == 0 ? 2 : 1, 128, 16);

    const long long units = (long long)P.nm * P.ntiles;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const int mi = (int)(u / P.ntiles), tile = (int)(u % P.ntiles);
        // 1. rows q = t, 128 + t: the 8 fields' S_f (rows 160..255 stay zero)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int q = 128 * h + t;
            if (q < kQ) {
                float row[16];
#pragma unroll
                for (int z = 0; z < 8; z++) {
                    const float2 v = P.sf[((long long)(2 * mi + z) * P.ntiles + tile) * kQ + q];
                    row[z] = v.x;
                    row[8 + z] = v.y;
                }
                put_row<KIND, 16>(af_hi + h * LY::blk, af_lo + h * LY::blk, t, LY::rb, row);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (t == 0) {
            fence_after();
            for (int h = 0; h < 2; h++)
                mma3<KIND>(tmem + 16 * h, smem_addr(af_hi + h * LY::blk), smem_addr(af_lo + h * LY::blk),
                           smem_addr(smem + LY::bf), smem_addr(smem + LY::bf + 16 * LY::rb), 8 * LY::rb, 8 * LY::rb,
                           LY::ks, id);
            mma_commit(bar);
        }
        bool ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();

        // 2. spectra of this thread's rows; their squared magnitudes for the mirrors
        float v[2][16];
        tmem_ld16(tmem + lane_base, v[0]);
        tmem_ld16(tmem + lane_base + 16, v[1]);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int q = 128 * h + t;
            if (q < kQ)
#pragma unroll
                for (int kz = 0; kz < 8; kz++) mag[q * 8 + kz] = __fmaf_rn(v[h][2 * kz], v[h][2 * kz], v[h][2 * kz + 1] * v[h][2 * kz + 1]);
        }
        __syncthreads();

        // 3. decisions; the kept bins are the inverse's operand
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int q = 128 * h + t;
            if (q < kQ) {
                const int kxi = q >> 5, ky = q & 31, kyr = (40 - ky) & 31;
                const int qm = (4 - kxi) * 32 + kyr;
                float row[16];
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    const int kzr = (10 - kz) & 7;
                    const bool keep = keep_pair(mag[q * 8 + kz], mag[qm * 8 + kzr], P.t2f) ||
                                      (kxi == 2 && kz == kzr && ky == kyr);
                    row[kz] = keep ? v[h][2 * kz] : 0.f;
                    row[8 + kz] = keep ? v[h][2 * kz + 1] : 0.f;
                }
                put_row<KIND, 16>(ai_hi + h * LY::blk, ai_lo + h * LY::blk, t, LY::rb, row);
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (t == 0) {
            fence_after();
            for (int h = 0; h < 2; h++)
                mma3<KIND>(tmem + 32 + 16 * h, smem_addr(ai_hi + h * LY::blk), smem_addr(ai_lo + h * LY::blk),
                           smem_addr(smem + LY::bi), smem_addr(smem + LY::bi + 16 * LY::rb), 8 * LY::rb, 8 * LY::rb,
                           LY::ks, id);
            mma_commit(bar);
        }
        ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();

        // 4. the four slices of each row
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float w[16];
            tmem_ld16(tmem + lane_base + 32 + 16 * h, w);
            const int q = 128 * h + t;
            if (q < kQ) {
                float2 *dst = P.rz + ((long long)mi * P.ntiles + tile) * 4 * kQ + q;
#pragma unroll
                for (int sl = 0; sl < 4; sl++) dst[sl * kQ] = make_float2(w[2 * sl], w[2 * sl + 1]);
            }
        }
        fence_before();
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

// ---------------------------------------------------------------------------
// Decode: Y and X inverse and overlap-add of 24 spatial tiles of one output
// field per CTA iteration. Output field 2k + j sums slice j of Z tile k and
// slice 4 + j of Z tile k - 2 (transform_pal_3d.cpp:214-215); the Y inverse
// gives its own-parity rows (y = y0 + 2 i), the X inverse its 16 samples,
// (2/4096) Re(sum over kx = 2..6), the conjugate bins kx = 10..14 of the
// reference's c2r folded into the factor 2 (transform_pal_3d.cpp:205-240).
// Each (tileY, tileX) parity class writes its own plane, as in the plain
// form.
// ---------------------------------------------------------------------------
template <int KIND>
struct YXLayout {
    static constexpr int eb = Split<KIND>::eb;
    static constexpr int rby = 64 * eb;     // Y inverse rows: 32 re + 32 im
    static constexpr int rbx = 16 * eb;     // X inverse rows: 5 kx re/im (+6 zero)
    static constexpr int ax_blk = 128 * rbx;
    static constexpr int ay = 0;                        // [split][128 rows]
    // the X operand reuses the Y operand's space (written once the Y MMAs are
    // complete; its pad columns 10..15 are zeroed with every write)
    static constexpr int ax = ay;                       // [split][3 blocks][128 rows]
    static_assert(2 * 3 * ax_blk <= 2 * 128 * rby, "X operand fits the Y operand's space");
    static constexpr int by = ay + 2 * 128 * rby;       // [y0][split][32 rows]
    static constexpr int bx = by + 2 * 2 * 32 * rby;    // [split][16 rows]
    static constexpr int bar = bx + ((2 * 16 * rbx + 1023) & ~1023);
    static constexpr int bytes = bar + 64;
    static constexpr int ksy = rby / 32;
    static constexpr int ksx = rbx / 32;
};

template <int KIND>
__global__ void __launch_bounds__(kThreads) tc3_yx_kernel(Params P)
{
    using LY = YXLayout<KIND>;
    using SP = Split<KIND>;
    constexpr int eb = LY::eb;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + LY::bar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + LY::bar + 8);
    const int t = threadIdx.x, warp = t >> 5;

    copy_image(smem + LY::by, P.byi, 2 * 2 * 32 * LY::rby);
    copy_image(smem + LY::bx, P.bxi, 2 * 16 * LY::rbx);
    for (int o = t * 16; o < 2 * 128 * LY::rby; o += kThreads * 16) *reinterpret_cast<uint4 *>(smem + LY::ay + o) = uint4{0, 0, 0, 0};
    if (t == 0) bar_init(bar);
    if (warp == 0) tmem_alloc(tslot, 128);   // Y inverse: columns 0..31, X inverse: 32..79
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    uint32_t phase = 0;
    uint8_t *ay_hi = smem + LY::ay, *ay_lo = smem + LY::ay + 128 * LY::rby;
    uint8_t *ax_hi = smem + LY::ax, *ax_lo = smem + LY::ax + 3 * LY::ax_blk;

    const int groups = (P.ntiles + kTilesPerUnit - 1) / kTilesPerUnit;
    const int units = P.nout * groups;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const int fo = u / groups;
        const int tile0 = (u % groups) * kTilesPerUnit;
        const int k = fo >> 1, j = fo & 1;
        const int f = 2 * (P.frame0 + k) + j;
        const int y0 = (((f & 1) ^ P.swap) - P.tileY0) & 1;   // every tileY has tileY0's parity

        // 1. Y inverse operand, row t = (tile, kx): R = slice j of Z tile k + slice 4 + j of Z tile k - 2
        if (t < kYRows) {
            const int ft = t / 5, kxi = t % 5;
            const int tile = tile0 + ft;
            if (tile < P.ntiles) {
                const float4 *ra = reinterpret_cast<const float4 *>(
                    P.rz + (((long long)(k + 2) * P.ntiles + tile) * 4 + j) * kQ + kxi * 32);
                const float4 *rb = reinterpret_cast<const float4 *>(
                    P.rz + (((long long)k * P.ntiles + tile) * 4 + 2 + j) * kQ + kxi * 32);
                float row[64];
#pragma unroll
                for (int c = 0; c < 16; c++) {   // two ky per float4
                    const float4 a = ra[c], b = rb[c];
                    row[2 * c] = a.x + b.x;
                    row[32 + 2 * c] = a.y + b.y;
                    row[2 * c + 1] = a.z + b.z;
                    row[33 + 2 * c] = a.w + b.w;
                }
                put_row<KIND, 64>(ay_hi, ay_lo, t, LY::rby, row);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (t == 0) {
            fence_after();
            const uint8_t *byh = smem + LY::by + (2 * y0) * 32 * LY::rby;
            mma3<KIND>(tmem, smem_addr(ay_hi), smem_addr(ay_lo), smem_addr(byh), smem_addr(byh + 32 * LY::rby),
                       8 * LY::rby, 8 * LY::rby, LY::ksy, idesc(KIND == 0 ? 2 : 1, 128, 32));
            mma_commit(bar);
        }
        bool ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();

        // 2. rows i of (tile, kx) -> X inverse operand rows (tile, i), columns kx re/im
        {
            float g0[16], g1[16];
            tmem_ld16(tmem + lane_base, g0);
            tmem_ld16(tmem + lane_base + 16, g1);
            if (t < kYRows) {
                const int ft = t / 5, kxi = t % 5;
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int R = ft * 16 + i;
                    const float re = i < 8 ? g0[2 * i] : g1[2 * i - 16];
                    const float im = i < 8 ? g0[2 * i + 1] : g1[2 * i - 15];
                    uint8_t *h = ax_hi + (R >> 7) * LY::ax_blk, *l = ax_lo + (R >> 7) * LY::ax_blk;
                    SP::put(h, l, elem_off(R & 127, 2 * kxi, eb, LY::rbx), re);
                    SP::put(h, l, elem_off(R & 127, 2 * kxi + 1, eb, LY::rbx), im);
                    if (kxi == 0)   // pad columns 10..15 (this space held the Y operand)
#pragma unroll
                        for (int c = 10; c < 16; c++) SP::put(h, l, elem_off(R & 127, c, eb, LY::rbx), 0.f);
                }
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (t == 0) {
            fence_after();
            for (int b = 0; b < 3; b++)
                mma3<KIND>(tmem + 32 + 16 * b, smem_addr(ax_hi + b * LY::ax_blk), smem_addr(ax_lo + b * LY::ax_blk),
                           smem_addr(smem + LY::bx), smem_addr(smem + LY::bx + 16 * LY::rbx), 8 * LY::rbx,
                           8 * LY::rbx, LY::ksx, idesc(KIND == 0 ? 2 : 1, 128, 16));
            mma_commit(bar);
        }
        ok = bar_wait(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (t == 0) atomicExch(P.err, 1);
            break;
        }
        fence_after();

        // 3. 16 samples of row (tile, i) into the tile's parity-class plane
        for (int b = 0; b < 3; b++) {
            float o[16];
            tmem_ld16(tmem + lane_base + 32 + 16 * b, o);
            const int R = 128 * b + t;
            const int tile = tile0 + (R >> 4), i = R & 15;
            if (tile < P.ntiles) {
                const int tx = tile % P.ntx, ty = tile / P.ntx;
                const int tileX = P.tileX0 + 8 * tx, tileY = P.tileY0 + 16 * ty;
                const int L = tileY + y0 + 2 * i;
                if (L >= P.fafl && L <= P.lafl) {
                    const int cls = ((ty & 1) << 1) | (tx & 1);
                    float *dst = P.partial + (long long)cls * P.part_class_stride +
                                 (long long)(P.out_field0 + fo) * P.part_field_stride +
                                 (long long)((L >> 1) - P.fl_lo) * P.part_row_stride - P.avs;
                    // interior tiles: tileX - avs is a multiple of 8, so with
                    // 4-float strides and a 16-byte base the row is 32-byte aligned
                    const bool vec = ((P.part_row_stride | P.part_field_stride | P.part_class_stride) & 3) == 0 &&
                                     (reinterpret_cast<uintptr_t>(P.partial) & 15) == 0 && tileX >= P.avs &&
                                     tileX + 16 <= P.ave;
                    if (vec) {
                        float4 *d4 = reinterpret_cast<float4 *>(dst + tileX);
#pragma unroll
                        for (int q = 0; q < 4; q++) d4[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
                    } else {
#pragma unroll
                        for (int x = 0; x < 16; x++) {
                            const int X = tileX + x;
                            if (X >= P.avs && X < P.ave) dst[X] = o[x];
                        }
                    }
                }
            }
        }
        fence_before();
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
// Host: coefficient images
// ---------------------------------------------------------------------------
static double rc_window(int n, int N) { return 0.5 - (0.5 * cos((2 * M_PI * (n + 0.5)) / N)); }

static float tf32_rna(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    memcpy(&f, &u, 4);
    return f;
}

static uint16_t bf16_rn(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

static float bf16_val(uint16_t h)
{
    const uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Write the (hi, lo) split of matrix M (rows x K, row-major doubles) as two
// operand images.
static void put_image(std::vector<uint8_t> &img, size_t off_hi, size_t off_lo, const std::vector<double> &M, int rows,
                      int K, int variant)
{
    const int eb = variant == 0 ? 4 : 2;
    const int rb = K * eb;
    for (int r = 0; r < rows; r++)
        for (int k = 0; k < K; k++) {
            const double v = M[(size_t)r * K + k];
            const uint32_t o = elem_off(r, k, eb, rb);
            if (variant == 0) {
                const float h = tf32_rna((float)v);
                const float l = tf32_rna((float)(v - (double)h));
                memcpy(&img[off_hi + o], &h, 4);
                memcpy(&img[off_lo + o], &l, 4);
            } else {
                const uint16_t h = bf16_rn((float)v);
                const uint16_t l = bf16_rn((float)(v - (double)bf16_val(h)));
                memcpy(&img[off_hi + o], &h, 2);
                memcpy(&img[off_lo + o], &l, 2);
            }
        }
}

// B_X [16 x 16]: row 2k + c (kx = k + 2), column x: w_x(x) (cos th, -sin th), th = 2 pi kx x / 16
static std::vector<double> matrix_x()
{
    std::vector<double> M(16 * 16, 0.0);
    for (int k = 0; k < 5; k++)
        for (int x = 0; x < 16; x++) {
            const double th = 2.0 * M_PI * (k + 2) * x / 16.0, w = rc_window(x, 16);
            M[(2 * k) * 16 + x] = w * cos(th);
            M[(2 * k + 1) * 16 + x] = -w * sin(th);
        }
    return M;
}

// B_Y [64 x 32] for row parity y0: row 2 ky + c, columns re(i), im(i);
// frame line y = y0 + 2 i, ph = 2 pi ky y / 32
static std::vector<double> matrix_y(int y0)
{
    std::vector<double> M(64 * 32, 0.0);
    for (int ky = 0; ky < 32; ky++)
        for (int i = 0; i < 16; i++) {
            const int y = y0 + 2 * i;
            const double ph = 2.0 * M_PI * ky * y / 32.0, w = rc_window(y, 32);
            M[(2 * ky) * 32 + i] = w * cos(ph);
            M[(2 * ky) * 32 + 16 + i] = w * sin(ph);
            M[(2 * ky + 1) * 32 + i] = -w * sin(ph);
            M[(2 * ky + 1) * 32 + 16 + i] = w * cos(ph);
        }
    return M;
}

// B_Z [16 x 16]: row 2 kz + c, columns re(z), im(z); ph = 2 pi kz z / 8
static std::vector<double> matrix_z()
{
    std::vector<double> M(16 * 16, 0.0);
    for (int kz = 0; kz < 8; kz++)
        for (int z = 0; z < 8; z++) {
            const double ph = 2.0 * M_PI * kz * z / 8.0, w = rc_window(z, 8);
            M[(2 * kz) * 16 + z] = w * cos(ph);
            M[(2 * kz) * 16 + 8 + z] = w * sin(ph);
            M[(2 * kz + 1) * 16 + z] = -w * sin(ph);
            M[(2 * kz + 1) * 16 + 8 + z] = w * cos(ph);
        }
    return M;
}

// B_Zi [16 x 16]: rows 2 s + c for the slices z_s = 0, 1, 4, 5 (rows 8..15
// zero), columns re(kz), im(kz); exp(+i ph), ph = 2 pi kz z_s / 8
static std::vector<double> matrix_zi()
{
    static const int zs[4] = {0, 1, 4, 5};
    std::vector<double> M(16 * 16, 0.0);
    for (int sl = 0; sl < 4; sl++)
        for (int kz = 0; kz < 8; kz++) {
            const double ph = 2.0 * M_PI * kz * zs[sl] / 8.0;
            M[(2 * sl) * 16 + kz] = cos(ph);
            M[(2 * sl) * 16 + 8 + kz] = -sin(ph);
            M[(2 * sl + 1) * 16 + kz] = sin(ph);
            M[(2 * sl + 1) * 16 + 8 + kz] = cos(ph);
        }
    return M;
}

// B_Yi [32 x 64] for row parity y0: rows 2 i + c (frame line y = y0 + 2 i),
// columns re(ky), im(ky); exp(+i ph), ph = 2 pi ky y / 32
static std::vector<double> matrix_yi(int y0)
{
    std::vector<double> M(32 * 64, 0.0);
    for (int i = 0; i < 16; i++)
        for (int ky = 0; ky < 32; ky++) {
            const double ph = 2.0 * M_PI * ky * (y0 + 2 * i) / 32.0;
            M[(2 * i) * 64 + ky] = cos(ph);
            M[(2 * i) * 64 + 32 + ky] = -sin(ph);
            M[(2 * i + 1) * 64 + ky] = sin(ph);
            M[(2 * i + 1) * 64 + 32 + ky] = cos(ph);
        }
    return M;
}

// B_Xi [16 x 16]: row x, columns kx re/im (10..15 zero): (2/4096) (cos th, -sin th), th = 2 pi kx x / 16
static std::vector<double> matrix_xi()
{
    std::vector<double> M(16 * 16, 0.0);
    for (int x = 0; x < 16; x++)
        for (int k = 0; k < 5; k++) {
            const double th = 2.0 * M_PI * (k + 2) * x / 16.0;
            M[x * 16 + 2 * k] = (2.0 / 4096.0) * cos(th);
            M[x * 16 + 2 * k + 1] = -(2.0 / 4096.0) * sin(th);
        }
    return M;
}

// Operand images of one variant: per stage [split] (the Y stages [y0][split]).
struct Images {
    std::vector<uint8_t> stage[6];   // 0 X, 1 Y, 2 Z forward; 3 Z, 4 Y, 5 X inverse
};

static Images build_images(int variant)
{
    const int eb = variant == 0 ? 4 : 2;
    Images im;
    const int rows[6] = {16, 64, 16, 16, 32, 16}, K[6] = {16, 32, 16, 16, 64, 16};
    for (int st = 0; st < 6; st++) {
        const size_t one = (size_t)rows[st] * K[st] * eb;
        const bool per_y0 = (st == 1 || st == 4);
        im.stage[st].assign((per_y0 ? 4 : 2) * one, 0);
        for (int y0 = 0; y0 < (per_y0 ? 2 : 1); y0++) {
            const std::vector<double> M = st == 0 ? matrix_x() : st == 1 ? matrix_y(y0) : st == 2 ? matrix_z()
                                        : st == 3 ? matrix_zi() : st == 4 ? matrix_yi(y0) : matrix_xi();
            put_image(im.stage[st], (2 * y0) * one, (2 * y0 + 1) * one, M, rows[st], K[st], variant);
        }
    }
    return im;
}

struct DeviceState {
    uint8_t *img[2] = {nullptr, nullptr};   // per variant: the six stages back to back
    size_t off[2][6] = {};
    float2 *sf = nullptr, *rz = nullptr;
    size_t sf_bytes = 0, rz_bytes = 0;
    int *err = nullptr;
    bool attrs = false;
};

static std::mutex g_mu;
static DeviceState g_dev[64];

static int fail(const std::string &what, int code)
{
    chd::detail::set_last_error("chromadec_gb300: " + what);
    return code;
}

static int grow(float2 *&buf, size_t &have, size_t need)
{
    if (have >= need) return 0;
    if (buf) {
        cudaDeviceSynchronize();
        cudaFree(buf);
    }
    buf = nullptr;
    have = 0;
    if (cudaMalloc(&buf, need) != cudaSuccess) return fail("tensor-core form: cudaMalloc", CHDG_E_OOM);
    have = need;
    return 0;
}

// Images, error flag, kernel attributes and scratch of the calling thread's
// device (under g_mu); fills the operand pointers of P.
static int prepare(int variant, size_t sf_need, size_t rz_need, Params &P, int &dev)
{
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail("tensor-core form: no CUDA device", CHDG_E_CUDA);
    DeviceState &D = g_dev[dev];
    if (!D.img[variant]) {
        const Images im = build_images(variant);
        std::vector<uint8_t> all;
        for (int st = 0; st < 6; st++) {
            D.off[variant][st] = all.size();
            all.insert(all.end(), im.stage[st].begin(), im.stage[st].end());
        }
        if (cudaMalloc(&D.img[variant], all.size()) != cudaSuccess) return fail("tensor-core form: cudaMalloc", CHDG_E_OOM);
        if (cudaMemcpy(D.img[variant], all.data(), all.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail("tensor-core form: upload", CHDG_E_CUDA);
    }
    if (!D.err) {
        if (cudaMalloc(&D.err, sizeof(int)) != cudaSuccess || cudaMemset(D.err, 0, sizeof(int)) != cudaSuccess)
            return fail("tensor-core form: cudaMalloc", CHDG_E_OOM);
    }
    if (const int rc = grow(D.sf, D.sf_bytes, sf_need); rc != 0) return rc;
    if (rz_need)
        if (const int rc = grow(D.rz, D.rz_bytes, rz_need); rc != 0) return rc;
    if (!D.attrs) {
        cudaFuncSetAttribute(tc3_xy_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, XYLayout<0>::bytes);
        cudaFuncSetAttribute(tc3_xy_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, XYLayout<1>::bytes);
        cudaFuncSetAttribute(tc3_z_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, ZLayout<0>::bytes);
        cudaFuncSetAttribute(tc3_z_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ZLayout<1>::bytes);
        cudaFuncSetAttribute(tc3_zd_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, ZDLayout<0>::bytes);
        cudaFuncSetAttribute(tc3_zd_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ZDLayout<1>::bytes);
        cudaFuncSetAttribute(tc3_yx_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, YXLayout<0>::bytes);
        cudaFuncSetAttribute(tc3_yx_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, YXLayout<1>::bytes);
        D.attrs = true;
    }
    const uint8_t *b = D.img[variant];
    P.bx = b + D.off[variant][0];
    P.by = b + D.off[variant][1];
    P.bz = b + D.off[variant][2];
    P.bzi = b + D.off[variant][3];
    P.byi = b + D.off[variant][4];
    P.bxi = b + D.off[variant][5];
    P.sf = D.sf;
    P.rz = D.rz;
    P.err = D.err;
    return 0;
}

static void tile_grid(Params &P, int avs, int ave, int fafl, int lafl)
{
    // transform_pal_3d.cpp:151-153
    P.tileX0 = avs - 8;
    P.ntx = (ave - P.tileX0 + 7) / 8;
    P.tileY0 = fafl - 16;
    P.nty = (lafl - P.tileY0) / 16 + 1;
    P.ntiles = P.ntx * P.nty;
}

static int sm_count(int dev)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <typename K>
static void launch(K kernel, long long work, int per_sm, int sms, int smem, cudaStream_t s, const Params &P)
{
    const int grid = (int)std::min<long long>(work, (long long)per_sm * sms);
    if (grid > 0) kernel<<<grid, kThreads, smem, s>>>(P);
}

static void launch_xy(int variant, const Params &P, int sms, cudaStream_t s)
{
    const long long units = (long long)P.nf * ((P.ntiles + kTilesPerUnit - 1) / kTilesPerUnit);
    if (variant == 0) launch(tc3_xy_kernel<0>, units, 2, sms, XYLayout<0>::bytes, s, P);
    else launch(tc3_xy_kernel<1>, units, 4, sms, XYLayout<1>::bytes, s, P);
}

}  // namespace tc

// The tensor-core form's transform stage of an engine decode: frames
// [frame_begin, frame_end) of T into its overlap-class planes, in chunks of
// up to 64 frames (each with its 2-frame look-behind of Z tiles and the
// fields they span). Uniform threshold only.
int tc3_transform(const T3Params &T, int field_height, int variant, cudaStream_t s)
{
    using namespace tc;
    if (variant < 0 || variant > 1 || T.thr_table != nullptr || T.frame_t2 != nullptr || T.field_ptrs != nullptr)
        return fail("tensor-core form: uniform threshold on one capture buffer only", CHDG_E_UNSUPPORTED);
    constexpr int kChunk = 64;
    Params P{};
    P.fields = T.fields;
    P.field_stride = T.field_stride;
    P.field_base = T.field_base;
    P.nfields = T.nfields;
    P.fw = T.fw;
    P.fh = field_height;
    P.fafl = T.fafl;
    P.lafl = T.lafl;
    P.black = T.black;
    P.swap = T.swap;
    tile_grid(P, T.avs, T.ave, T.fafl, T.lafl);
    P.t2f = T.t2f;
    P.partial = T.partial;
    P.part_class_stride = T.part_class_stride;
    P.part_field_stride = T.part_field_stride;
    P.part_row_stride = T.part_row_stride;
    P.fl_lo = T.fl_lo;
    P.avs = T.avs;
    P.ave = T.ave;
    const int maxc = std::min(kChunk, T.frame_end - T.frame_begin);
    const size_t sf_need = (size_t)(2 * (maxc + 2) + 6) * P.ntiles * kQ * sizeof(float2);
    const size_t rz_need = (size_t)(maxc + 2) * P.ntiles * 4 * kQ * sizeof(float2);
    int dev = 0;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (const int rc = prepare(variant, sf_need, rz_need, P, dev); rc != 0) return rc;
    }
    const int sms = sm_count(dev);
    for (int c0 = T.frame_begin; c0 < T.frame_end; c0 += kChunk) {
        const int c1 = std::min(T.frame_end, c0 + kChunk);
        P.nm = (c1 - c0) + 2;         // Z tiles c0 - 2 .. c1 - 1
        P.f_begin = 2 * (c0 - 2);
        P.nf = 2 * P.nm + 6;
        P.frame0 = c0;
        P.nout = 2 * (c1 - c0);
        P.out_field0 = 2 * (c0 - T.frame_begin);
        launch_xy(variant, P, sms, s);
        const long long zd_units = (long long)P.nm * P.ntiles;
        const long long yx_units = (long long)P.nout * ((P.ntiles + kTilesPerUnit - 1) / kTilesPerUnit);
        // CTAs per SM: shared memory and tensor memory (512 columns) allow
        if (variant == 0) {
            launch(tc3_zd_kernel<0>, zd_units, 5, sms, ZDLayout<0>::bytes, s, P);
            launch(tc3_yx_kernel<0>, yx_units, 2, sms, YXLayout<0>::bytes, s, P);
        } else {
            launch(tc3_zd_kernel<1>, zd_units, 8, sms, ZDLayout<1>::bytes, s, P);
            launch(tc3_yx_kernel<1>, yx_units, 4, sms, YXLayout<1>::bytes, s, P);
        }
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("tensor-core form: launch: ") + cudaGetErrorString(e), CHDG_E_CUDA);
    return 0;
}

int tc3_launches_per_frames(int frames) { return 3 * ((frames + 63) / 64); }

}  // namespace tpal

using namespace tpal::tc;

#pragma GCC visibility push(default)
extern "C" {

int chdg_tc3d_operand(int32_t variant, int32_t stage, int32_t y0, int32_t split, void *out, size_t bytes)
{
    if (variant < 0 || variant > 1 || stage < 0 || stage > 5 || y0 < 0 || y0 > 1 || split < 0 || split > 1 || !out)
        return fail("chdg_tc3d_operand: bad argument", CHDG_E_INVALID_ARG);
    const Images im = build_images(variant);
    const std::vector<uint8_t> &src = im.stage[stage];
    const bool per_y0 = (stage == 1 || stage == 4);
    const size_t one = src.size() / (per_y0 ? 4 : 2);
    const size_t off = (per_y0 ? (size_t)(2 * y0 + split) : (size_t)split) * one;
    if (bytes < one) return fail("chdg_tc3d_operand: buffer too small", CHDG_E_INVALID_ARG);
    memcpy(out, src.data() + off, one);
    return (int)one;
}

int chdg_tc3d_spectra(const chdg_geometry *g, int32_t variant, const uint16_t *d_fields, int64_t field_stride,
                      int32_t nfields, int32_t m_begin, int32_t m_end, void *d_spec, void *stream)
{
    if (!g || !d_fields || !d_spec || variant < 0 || variant > 1 || m_end <= m_begin || nfields <= 0 ||
        field_stride < (int64_t)g->field_width * g->field_height)
        return fail("chdg_tc3d_spectra: bad argument", CHDG_E_INVALID_ARG);
    Params P{};
    P.fields = d_fields;
    P.field_stride = field_stride;
    P.field_base = 0;
    P.nfields = nfields;
    P.fw = g->field_width;
    P.fh = g->field_height;
    P.fafl = g->first_active_frame_line;
    P.lafl = g->last_active_frame_line;
    P.black = g->black;
    P.swap = 0;
    tile_grid(P, g->active_start, g->active_end, g->first_active_frame_line, g->last_active_frame_line);
    P.nm = m_end - m_begin;
    P.f_begin = 2 * m_begin;
    P.nf = 2 * P.nm + 6;
    P.spec = (float2 *)d_spec;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        const size_t sf_need = (size_t)P.nf * P.ntiles * kQ * sizeof(float2);
        if (const int rc = prepare(variant, sf_need, 0, P, dev); rc != 0) return rc;
    }
    const int sms = sm_count(dev);
    launch_xy(variant, P, sms, s);
    const long long zblocks = ((long long)P.nm * P.ntiles * kQ + 127) / 128;
    if (variant == 0) launch(tc3_z_kernel<0>, zblocks, 8, sms, ZLayout<0>::bytes, s, P);
    else launch(tc3_z_kernel<1>, zblocks, 8, sms, ZLayout<1>::bytes, s, P);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("chdg_tc3d_spectra: launch: ") + cudaGetErrorString(e), CHDG_E_CUDA);
    return 0;
}

int chdg_tc3d_sync(void *stream)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail("chdg_tc3d_sync: no CUDA device", CHDG_E_CUDA);
    const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return fail(std::string("chdg_tc3d_sync: ") + cudaGetErrorString(e), CHDG_E_CUDA);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_dev[dev].err) return 0;
    int flag = 0;
    if (cudaMemcpy(&flag, g_dev[dev].err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail("chdg_tc3d_sync: read flag", CHDG_E_CUDA);
    if (flag) {
        cudaMemset(g_dev[dev].err, 0, sizeof(int));
        return fail("chdg_tc3d_sync: a tensor-core completion wait ran out", CHDG_E_CUDA);
    }
    return 0;
}

}  // extern "C"
#pragma GCC visibility pop
