// demod.cu -- PALcolour demodulation of Transform-PAL chroma and on-device
// H.273 quantise/pack, sm_103a.
//
// Follows PalColour::decodeField / detectBurst / decodeLine<double, true>
// (src/decoders/palcolour/palcolour.cpp:307-409, 456-646) and
// OutputWriter::convertLine / convertToFloat
// (src/output/output_writer.cpp:402-486, 670-727), restructured:
//
//  * 4fsc sampling makes the reference carrier exact: sin(2 pi i fSC/fs) is
//    {0, 1, 0, -1}[i mod 4] (the reference's double tables differ only by
//    ~1e-16 residues at the zeros). The burst sums therefore run in exact
//    integer arithmetic, the V-switch test is an exact int64 comparison, and
//    each FIR tap touches either the sine or the cosine products, never both.
//  * The chroma input is the sum of the transform's four overlap-class planes;
//    chroma lines outside the field's active lines and samples outside the
//    active window are zero, exactly like the reference's zero-initialised
//    chroma buffer and its blackLine substitution (palcolour.cpp:466-473).
//  * Y = composite - chroma, the rotated U/V and the output scaling are fused;
//    planes are written straight into the frame's [Y | Cb | Cr] layout.
//
//  * CHD_DEC_PAL_2D (partial == NULL): the same 2D FIR runs on the composite
//    rows themselves (decodeLine<uint16_t, false>) and luma is the composite
//    minus the chroma the Y filter extracts, resynthesised on the carrier.
//  * luma_nr_level > 0: doYNR (palcolour.cpp:412-449) -- the 25-tap
//    high-pass of each line's luma, cored to +-nr_y and subtracted -- after a
//    pre-pass that puts the block's luma lines in shared memory.
//  * Every output format of the ABI is packed here: yuv444p16/ps, rgb48
//    (interleaved, truncating), rgbs, gray16, grays.
//
// One block: 16 field lines (8 with yNR) of one output field, 256 threads; a
// work item produces 8 consecutive samples of one line from a register window
// of the four vertically combined chroma rows.
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "tpal_common.cuh"
#include "tpal_kernels.h"

namespace tpal {

__constant__ float cd_nrpal[25];     // doYNR high-pass (c_nrpal_b)
static bool g_demod_ready[64];

constexpr int kDemodThreads = 256;
constexpr int kPad = 8;
constexpr int kNrHalf = 12;              // half length of the yNR filter
// Field lines per block: 16 (a 6-line halo re-read per 16 lines), 8 with
// yNR, whose luma lines also live in shared memory.
__host__ __device__ constexpr int demod_lines(bool ynr) { return ynr ? 8 : 16; }

__device__ __forceinline__ int first_line(int fafl, int off) { return (fafl + 1 - off) / 2; }
__device__ __forceinline__ int last_line(int lafl, int off) { return ((lafl - off) / 2) + 1; }

__host__ __device__ __forceinline__ int demod_span(int avs, int ave) { return ((ave - (avs & ~3)) + 7) & ~7; }

// 4fsc reference carrier at sample x: sine {0, 1, 0, -1}, cosine {1, 0, -1, 0}.
__device__ __forceinline__ float carrier_sin(int x) { return (x & 1) ? ((x & 2) ? -1.f : 1.f) : 0.f; }
__device__ __forceinline__ float carrier_cos(int x) { return (x & 1) ? 0.f : ((x & 2) ? -1.f : 1.f); }

// The 2D FIR of one work item: PU, QU, PV, QV (and PY, QY from the luma
// taps when WITH_Y) for 8 samples from the 4 vertical combinations v.
// Taps b = 0..7 of the launch's filter (a filter of size 6, at PAL-M's
// sample rate, has zero taps at b = 7). swap: the reference's PAL-M tables
// (sine and cosine exchanged at fieldHeight 263, palcolour.cpp:158-173) make
// each P sum the other table's Q sum and vice versa: (PU, QU, PV, QV)
// become (QV, PV, QU, PU); the luma resynthesis is unchanged.
template <bool WITH_Y>
__device__ __forceinline__ void item_fir(const DemodParams &P, const float (&v)[4][22], float (&PU)[8], float (&QU)[8],
                                         float (&PV)[8], float (&QV)[8], float (&PY)[8], float (&QY)[8])
{
#pragma unroll
    for (int s = 0; s < 8; s++) {
        float PA = 0.f, PB = 0.f, QA = 0.f, QB = 0.f, PYs = 0.f, QYs = 0.f;
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int r = s + b + 7, l = s - b + 7;
            float sg[4];
#pragma unroll
            for (int k = 0; k < 4; k++) sg[k] = (b & 1) ? v[k][r] - v[k][l] : v[k][r] + v[k][l];
            const float A = __fmaf_rn(P.cfilt[b][1], sg[1], P.cfilt[b][0] * sg[0]);
            const float B = __fmaf_rn(P.cfilt[b][3], sg[3], P.cfilt[b][2] * sg[2]);
            float AY = 0.f;
            if (WITH_Y) AY = __fmaf_rn(P.yfilt[b][1], sg[1], P.yfilt[b][0] * sg[0]);
            switch ((s + b) & 3) {
            case 1: PA += A; PB += B; if (WITH_Y) PYs += AY; break;
            case 3: PA -= A; PB -= B; if (WITH_Y) PYs -= AY; break;
            case 0: QA += A; QB += B; if (WITH_Y) QYs += AY; break;
            default: QA -= A; QB -= B; if (WITH_Y) QYs -= AY; break;
            }
        }
        if (P.swap_carrier) {
            PU[s] = QA + PB;
            PV[s] = QA - PB;
            QU[s] = PA - QB;
            QV[s] = PA + QB;
        } else {
            PU[s] = PA + QB;
            PV[s] = PA - QB;
            QU[s] = QA - PB;
            QV[s] = QA + PB;
        }
        PY[s] = PYs;
        QY[s] = QYs;
    }
}

// Vertical combinations (palcolour.cpp:557-567 without the carrier):
//   v0 = c0, v1 = -c(-2) - c(+2), v2 = c(-1) - c(+1), v3 = -c(-3) + c(+3)
__device__ __forceinline__ void item_window(const float *rw, int SW, float (&v)[4][22])
{
#pragma unroll
    for (int q = 0; q < 22; q++) {
        v[0][q] = rw[3 * SW + q];
        v[1][q] = -rw[1 * SW + q] - rw[5 * SW + q];
        v[2][q] = rw[2 * SW + q] - rw[4 * SW + q];
        v[3][q] = -rw[q] + rw[6 * SW + q];
    }
}

// An integer-format code (H.273 Round(x) = Sign(x) * Floor(Abs(x) + 0.5),
// then the clamp, output_writer.cpp:52-76), zero + Round(v * (k_hi + k_lo)) for v = v_hi + v_lo,
// without FP32 rounding at the code's magnitude: the product is formed as
// p + e (p = v_hi k_hi rounded, e its error and the low-order terms), the
// nearest integer n of p split off exactly, and only the remainder
// (p - n) + e, below one in magnitude, rounded. zero is an integer, so
// zero + n + Floor(r + 1/2) is H.273's Round of the whole sum wherever that
// sum is non-negative; below zero both clamp to the bound lo >= 0. Returns
// the clamped code as a float (exact).
__device__ __forceinline__ float code_of(float zero, float v_hi, float v_lo, float k_hi, float k_lo, float lo, float hi)
{
    const float p = v_hi * k_hi;
    const float e = __fmaf_rn(v_hi, k_hi, -p) + __fmaf_rn(v_hi, k_lo, v_lo * k_hi);
    const float n = rintf(p);
    const float r = (p - n) + e;   // p - n is exact
    return fminf(fmaxf(zero + n + floorf(r + 0.5f), lo), hi);
}

// Pack one sample in the output format (OutputWriter::convertLine,
// convertToFloat, convertToFloatRGB; output_writer.cpp:402-486, 670-779).
// Luma arrives as Y - black = yb.hi + yb.lo (exact for the Transform kinds:
// an integer composite sample minus the FP32 chroma, by two-sum).
__device__ __forceinline__ void pack_sample(const DemodParams &P, void *out, long long frame, long long pix, df yb,
                                            float U, float V)
{
    const long long plane = (long long)P.out_w * P.out_h;
    const long long e = frame * P.out_frame_stride + pix;
    const float ey = (yb.hi + yb.lo) * P.ey_scale;
    switch (P.format) {
    case 0: {
        uint16_t *o = (uint16_t *)out;
        o[e] = (uint16_t)code_of(16.0f * 256.0f, yb.hi, yb.lo, P.qy_hi, P.qy_lo, P.y_lo, P.y_hi);
        o[e + plane] = (uint16_t)code_of(128.0f * 256.0f, U, 0.f, P.qcb_hi, P.qcb_lo, P.c_lo, P.c_hi);
        o[e + 2 * plane] = (uint16_t)code_of(128.0f * 256.0f, V, 0.f, P.qcr_hi, P.qcr_lo, P.c_lo, P.c_hi);
        break;
    }
    case 1: {
        float *o = (float *)out;
        o[e] = fminf(fmaxf(ey, P.y_lo), P.y_hi);
        o[e + plane] = fminf(fmaxf(U * P.ecb_scale, P.c_lo), P.c_hi);
        o[e + 2 * plane] = fminf(fmaxf(V * P.ecr_scale, P.c_lo), P.c_hi);
        break;
    }
    case 2: {   // interleaved R'G'B' 0..65535, truncating stores
        uint16_t *o = (uint16_t *)out + frame * P.out_frame_stride + 3 * pix;
        const float rY = fminf(fmaxf((yb.hi + yb.lo) * P.rgb_y_scale, 0.f), 65535.f);
        const float rU = U * P.rgb_uv_scale, rV = V * P.rgb_uv_scale;
        o[0] = (uint16_t)__float2uint_rz(fminf(fmaxf(__fmaf_rn(P.r_from_v, rV, rY), 0.f), 65535.f));
        o[1] = (uint16_t)__float2uint_rz(
            fminf(fmaxf(__fmaf_rn(P.g_from_v, rV, __fmaf_rn(P.g_from_u, rU, rY)), 0.f), 65535.f));
        o[2] = (uint16_t)__float2uint_rz(fminf(fmaxf(__fmaf_rn(P.b_from_u, rU, rY), 0.f), 65535.f));
        break;
    }
    case 3: {
        float *o = (float *)out;
        const float rU = U * P.rgb_uv_scale, rV = V * P.rgb_uv_scale;
        o[e] = fminf(fmaxf(__fmaf_rn(P.r_from_v, rV, ey), P.r_lo), P.r_hi);
        o[e + plane] = fminf(fmaxf(__fmaf_rn(P.g_from_v, rV, __fmaf_rn(P.g_from_u, rU, ey)), P.g_lo), P.g_hi);
        o[e + 2 * plane] = fminf(fmaxf(__fmaf_rn(P.b_from_u, rU, ey), P.b_lo), P.b_hi);
        break;
    }
    case 4:
        ((uint16_t *)out)[e] = (uint16_t)code_of(16.0f * 256.0f, yb.hi, yb.lo, P.qy_hi, P.qy_lo, P.y_lo, P.y_hi);
        break;
    default:
        ((float *)out)[e] = fminf(fmaxf(ey, P.y_lo), P.y_hi);
        break;
    }
}

// The three outputs of one sample in the units yuv444p16 (the quantised
// code, exact in FP32) or yuv444ps (E'Y, E'Cb, E'Cr) stores -- the
// arithmetic of pack_sample's cases 0 and 1.
__device__ __forceinline__ void yuv_values(const DemodParams &P, df yb, float U, float V, float &o0, float &o1,
                                           float &o2)
{
    if (P.format == 0) {
        o0 = code_of(16.0f * 256.0f, yb.hi, yb.lo, P.qy_hi, P.qy_lo, P.y_lo, P.y_hi);
        o1 = code_of(128.0f * 256.0f, U, 0.f, P.qcb_hi, P.qcb_lo, P.c_lo, P.c_hi);
        o2 = code_of(128.0f * 256.0f, V, 0.f, P.qcr_hi, P.qcr_lo, P.c_lo, P.c_hi);
    } else {
        o0 = fminf(fmaxf((yb.hi + yb.lo) * P.ey_scale, P.y_lo), P.y_hi);
        o1 = fminf(fmaxf(U * P.ecb_scale, P.c_lo), P.c_hi);
        o2 = fminf(fmaxf(V * P.ecr_scale, P.c_lo), P.c_hi);
    }
}

__device__ __forceinline__ void store_yuv(const DemodParams &P, void *out, long long e, long long plane, float o0,
                                          float o1, float o2)
{
    if (P.format == 0) {
        uint16_t *o = (uint16_t *)out;
        o[e] = (uint16_t)o0;
        o[e + plane] = (uint16_t)o1;
        o[e + 2 * plane] = (uint16_t)o2;
    } else {
        float *o = (float *)out;
        o[e] = o0;
        o[e + plane] = o1;
        o[e + 2 * plane] = o2;
    }
}

// 8 consecutive outputs of one plane at element e (a multiple of 4): two
// 8-byte stores (yuv444p16) or two 16-byte stores (yuv444ps)
__device__ __forceinline__ void store8(const DemodParams &P, void *out, long long e, const float (&a)[8])
{
    if (P.format == 0) {
        uint2 *o = reinterpret_cast<uint2 *>((uint16_t *)out + e);
        o[0] = make_uint2((uint32_t)a[0] | ((uint32_t)a[1] << 16), (uint32_t)a[2] | ((uint32_t)a[3] << 16));
        o[1] = make_uint2((uint32_t)a[4] | ((uint32_t)a[5] << 16), (uint32_t)a[6] | ((uint32_t)a[7] << 16));
    } else {
        float4 *o = reinterpret_cast<float4 *>((float *)out + e);
        o[0] = make_float4(a[0], a[1], a[2], a[3]);
        o[1] = make_float4(a[4], a[5], a[6], a[7]);
    }
}

// Double-float pieces of the burst normalisation (FP64 is scarce on this
// GPU and one lane per line waiting on it stalls the block).
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

// max(sqrt(pn^2 + qn^2), floor), the square root refined by one Newton step
__device__ __forceinline__ df burst_norm(float pn, float qn, float floor_v)
{
    const df s = df_add(two_prod(pn, pn), two_prod(qn, qn));
    df r = df_make(0.f);
    if (s.hi > 0.f) {
        const float x = __fsqrt_rn(s.hi);
        const df d = df_sub(s, two_prod(x, x));
        r = quick_two_sum(x, __fdiv_rn(d.hi, 2.0f * x));
    }
    if (r.hi > floor_v || (r.hi == floor_v && r.lo > 0.f)) return r;
    return df_make(floor_v);
}

// a / d for an exact float a
__device__ __forceinline__ df df_div_f(float a, df d)
{
    const float q1 = __fdiv_rn(a, d.hi);
    const df r = df_sub(df_sub(df_make(a), two_prod(q1, d.hi)), df_make(q1 * d.lo));
    return quick_two_sum(q1, __fdiv_rn(r.hi, d.hi));
}

__device__ __forceinline__ float df_round(df v) { return __fadd_rn(v.hi, v.lo); }

template <bool COMPOSITE, bool YNR>
__global__ void __launch_bounds__(kDemodThreads, 2) demod_kernel(const __grid_constant__ DemodParams P)
{
    constexpr int kDemodLines = demod_lines(YNR);
    constexpr int kRows = kDemodLines + 6;   // input lines fl0-3 .. fl0+L+2
    extern __shared__ float smem[];
    const int nblk_per_field = (P.fh + kDemodLines - 1) / kDemodLines;   // upper bound; invalid lines skip
    const int o = blockIdx.x / nblk_per_field;
    const int blk = blockIdx.x % nblk_per_field;
    if (o >= P.nout) return;
    const int f = P.field_begin + o;
    const int off = (f & 1) ^ P.swap;   // SourceField::getOffset
    const int fl_first = first_line(P.fafl, off);
    const int fl_last = last_line(P.lafl, off);
    const int fl0 = fl_first + blk * kDemodLines;
    if (fl0 >= fl_last) return;

    const int base4 = P.avs & ~3;                     // absolute sample of local index 0
    const int span = demod_span(P.avs, P.ave);        // samples covered by threads (multiple of 8)
    const int SW = span + 2 * kPad;                   // smem row length
    const int YW = span + 2 * kNrHalf;                // luma line length (yNR)
    float *ch = smem;                                  // [kRows][SW] rows fl0-3 .. fl0+L+2
    float *ys = smem + kRows * SW;                     // [kDemodLines][YW] luma before coring (yNR only)
    __shared__ float s_bp[kDemodLines], s_bq[kDemodLines], s_vsw[kDemodLines];

    // where this field's frame goes: the frame slot of the output array, or
    // (batches of captures) the frame's own pointer, absent for the black
    // gap frames between captures
    void *out_base = P.out;
    long long frame_slot = o >> 1;   // field_begin is even: fields 2k, 2k+1 form frame k
    if (P.frame_out != nullptr) {
        out_base = P.frame_out[f >> 1];
        frame_slot = 0;
        if (out_base == nullptr) return;
    }
    const uint16_t *field = field_at(P, f);
    if (field == nullptr) return;   // a black batch gap: nothing to write
    const int cols = P.ave - P.avs;

    // 1. input rows, zero outside the field's active lines: the summed
    //    overlap-class chroma planes (zero outside the active window, the
    //    reference's zero-initialised chroma buffer), or the composite
    //    itself for the PALcolour filter (blackLine = 0, palcolour.cpp:466-473).
    for (int idx = threadIdx.x; idx < kRows * SW; idx += blockDim.x) ch[idx] = 0.f;
    if (YNR)
        for (int idx = threadIdx.x; idx < kDemodLines * YW; idx += blockDim.x) ys[idx] = 0.f;
    __syncthreads();
    if (COMPOSITE) {
        for (int idx = threadIdx.x; idx < kRows * SW; idx += blockDim.x) {
            const int r = idx / SW, c = idx % SW;
            const int fl = fl0 - 3 + r;
            const int x = base4 - kPad + c;
            if (fl < fl_first || fl >= fl_last || x < 0 || x >= P.fw) continue;
            ch[idx] = (float)field[(long long)fl * P.fw + x];
        }
    } else {
        const float *part = P.partial + (long long)o * P.part_field_stride;
        const int c4 = cols >> 2;   // float4 per row (cols is a multiple of 4 when avs is)
        const bool vec = ((cols & 3) == 0) && ((P.part_row_stride & 3) == 0) && ((P.part_class_stride & 3) == 0) &&
                         ((P.part_field_stride & 3) == 0);
        if (vec) {
#pragma unroll 4
            for (int idx = threadIdx.x; idx < kRows * c4; idx += blockDim.x) {
                const int r = idx / c4, q = idx % c4;
                const int fl = fl0 - 3 + r;
                if (fl < fl_first || fl >= fl_last) continue;
                const float4 *src =
                    reinterpret_cast<const float4 *>(part + (long long)(fl - P.fl_lo) * P.part_row_stride) + q;
                const long long cs4 = P.part_class_stride >> 2;
                float4 a = __ldg(src), b = __ldg(src + cs4), c = __ldg(src + 2 * cs4), d = __ldg(src + 3 * cs4);
                float *dst = ch + r * SW + kPad + (P.avs - base4) + 4 * q;
                dst[0] = (a.x + b.x) + (c.x + d.x);
                dst[1] = (a.y + b.y) + (c.y + d.y);
                dst[2] = (a.z + b.z) + (c.z + d.z);
                dst[3] = (a.w + b.w) + (c.w + d.w);
            }
        } else {
            for (int idx = threadIdx.x; idx < kRows * cols; idx += blockDim.x) {
                const int r = idx / cols, c = idx % cols;
                const int fl = fl0 - 3 + r;
                if (fl < fl_first || fl >= fl_last) continue;
                const long long e = (long long)(fl - P.fl_lo) * P.part_row_stride + c;
                float v = 0.f;
                for (int k = 0; k < P.nclasses; k++) v += part[(long long)k * P.part_class_stride + e];
                ch[r * SW + kPad + (P.avs - base4) + c] = v;
            }
        }
    }

    // 2. burst detection: one warp per line (detectBurst, palcolour.cpp:344-409)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int ln = warp; ln < kDemodLines; ln += kDemodThreads / 32) {
        const int fl = fl0 + ln;
        long long Ps = 0, Qs = 0, POs = 0, QOs = 0;
        if (fl < fl_last) {
            auto px = [&](int line, int i) -> int {
                return (line < 0 || line >= P.fh) ? 0 : (int)field[(long long)line * P.fw + i];
            };
            for (int i = P.burst_start + lane; i < P.burst_end; i += 32) {
                const int d = 2 * px(fl, i) - px(fl - 2, i) - px(fl + 2, i);   // 4 * ((in0 - (in3+in4)/2) / 2)
                const int e = px(fl + 1, i) - px(fl - 1, i);                   // 2 * ((in2 - in1) / 2)
                switch (i & 3) {
                case 0: Qs += d; QOs += e; break;    // cosine +1
                case 1: Ps += d; POs += e; break;    // sine +1
                case 2: Qs -= d; QOs -= e; break;    // cosine -1
                default: Ps -= d; POs -= e; break;   // sine -1
                }
            }
        }
#pragma unroll
        for (int h = 16; h >= 1; h >>= 1) {
            Ps += __shfl_xor_sync(0xffffffffu, Ps, h);
            Qs += __shfl_xor_sync(0xffffffffu, Qs, h);
            POs += __shfl_xor_sync(0xffffffffu, POs, h);
            QOs += __shfl_xor_sync(0xffffffffu, QOs, h);
        }
        if (P.swap_carrier) {   // the PAL-M tables: the sine sums are the cosine sums and vice versa
            const long long t0 = Ps, t1 = POs;
            Ps = Qs;
            Qs = t0;
            POs = QOs;
            QOs = t1;
        }
        if (lane == 0) {
            // bp = P/(4 len), bpo = PO/(2 len): the V-switch test scaled by (4 len)^2
            const long long a = Ps - 2 * POs, b = Qs - 2 * QOs;
            const bool vpos = (a * a + b * b) < 2 * (Ps * Ps + Qs * Qs);
            // bp / max(|(bp, bq)|, 130000/128) with bp = pn / (8 len): the
            // 8 len cancels, leaving pn / max(|(pn, qn)|, 8 len 130000/128).
            // pn, qn are integers below 2^23 (exact in FP32); the rest runs
            // in double-float (about 2^-46), so the rounded results are the
            // double computation's.
            const float pn = (float)(Ps - 2 * QOs), qn = (float)(Qs + 2 * POs);
            const df n = burst_norm(pn, qn, 8.0f * (float)(P.burst_end - P.burst_start) * (130000.0f / 128.0f));
            const df nbp = df_div_f(pn, n), nbq = df_div_f(qn, n);
            s_bp[ln] = df_round(df_sub(df_mul_f(nbp, P.gain_cos), df_mul_f(nbq, P.gain_sin)));
            s_bq[ln] = df_round(df_add(df_mul_f(nbp, P.gain_sin), df_mul_f(nbq, P.gain_cos)));
            s_vsw[ln] = vpos ? 1.f : -1.f;
        }
    }
    __syncthreads();

    const int per_line = span / 8;

    // 3. yNR pre-pass: the block's luma lines (zero outside the active window)
    if (YNR) {
        for (int item = threadIdx.x; item < kDemodLines * per_line; item += blockDim.x) {
            const int t = item / per_line, seg = item % per_line;
            const int fl = fl0 + t;
            if (fl >= fl_last) continue;
            const int xl0 = seg * 8;
            const uint16_t *comp = field + (long long)fl * P.fw;
            float Yv[8];
            if (COMPOSITE) {
                float v[4][22];
                item_window(ch + t * SW + kPad + xl0 - 7, SW, v);
                float PU[8], QU[8], PV[8], QV[8], PY[8], QY[8];
                item_fir<true>(P, v, PU, QU, PV, QV, PY, QY);
#pragma unroll
                for (int s = 0; s < 8; s++) {
                    const int x = base4 + xl0 + s;
                    Yv[s] = (float)comp[x < P.fw ? x : P.fw - 1] -
                            2.0f * __fmaf_rn(PY[s], carrier_sin(x), QY[s] * carrier_cos(x));
                }
            } else {
#pragma unroll
                for (int s = 0; s < 8; s++) {
                    const int x = base4 + xl0 + s;
                    Yv[s] = (float)comp[x < P.fw ? x : P.fw - 1] - ch[(t + 3) * SW + kPad + xl0 + s];
                }
            }
#pragma unroll
            for (int s = 0; s < 8; s++) {
                const int x = base4 + xl0 + s;
                if (x >= P.avs && x < P.ave) ys[t * YW + kNrHalf + xl0 + s] = Yv[s];
            }
        }
        __syncthreads();
    }

    // 4. 2D FIR + rotation + pack; work item = (line, 8-sample segment).
    // Sample s of an item is output pixel 8 seg + s - xoff. For yuv444p16 /
    // yuv444ps with 4-element-aligned rows, planes and frames, a lane stores
    // pixels 8 seg .. 8 seg + 7 with vector stores: its samples xoff..7 and
    // (xoff = 1) the next lane's sample 0, passed by a shuffle; edges and the
    // other formats store per sample. Every lane runs every round, so the
    // shuffles see the whole warp.
    const int total = kDemodLines * per_line;
    const int xoff = P.avs - base4;
    const int aw = P.ave - P.avs;
    const long long plane = (long long)P.out_w * P.out_h;
    const bool vout = (P.format == 0 || P.format == 1) && xoff <= 1 && ((P.out_w | P.left_pad) & 3) == 0 &&
                      (P.out_frame_stride & 3) == 0 && (reinterpret_cast<uintptr_t>(out_base) & 15) == 0;
    for (int ib = 0; ib < total; ib += blockDim.x) {
        const int item = ib + threadIdx.x;
        const int t = item / per_line;
        const int seg = item % per_line;
        const int fl = fl0 + t;
        const bool live = item < total && fl < fl_last;
        float o0[8], o1[8], o2[8];
        long long rowpix = 0;
        if (live) {
            const int xl0 = seg * 8;   // local index of the first sample (absolute base4 + xl0, a multiple of 4)
            // the composite samples luma needs, loaded before the FIR so their
            // latency hides behind it
            const uint16_t *comp = field + (long long)fl * P.fw;
            float cv[8];
#pragma unroll
            for (int s = 0; s < 8; s++) {
                const int x = base4 + xl0 + s;
                cv[s] = (float)comp[x < P.fw ? x : P.fw - 1];
            }
            float v[4][22];
            item_window(ch + t * SW + kPad + xl0 - 7, SW, v);
            float PU[8], QU[8], PV[8], QV[8], PY[8], QY[8];
            item_fir<COMPOSITE && !YNR>(P, v, PU, QU, PV, QV, PY, QY);

            const float bp = s_bp[t], bq = s_bq[t], vsw = s_vsw[t];
            const int orow = P.top_pad + 2 * fl + off - P.fafl;
            rowpix = (long long)orow * P.out_w + P.left_pad;
#pragma unroll
            for (int s = 0; s < 8; s++) {
                const int x = base4 + xl0 + s;
                df yb;   // Y - black
                const float cb = cv[s] - (float)P.black;   // exact: an integer sample
                if (YNR) {
                    // doYNR: a = sum_i b_i Y[x + 12 - i], cored to +-nr_y, subtracted
                    const float *yl = ys + t * YW + kNrHalf + xl0 + s;
                    float a = 0.f;
#pragma unroll
                    for (int i = 0; i < 25; i++) a = __fmaf_rn(cd_nrpal[i], yl[kNrHalf - i], a);
                    a = fminf(fmaxf(a, -P.nr_y), P.nr_y);
                    yb = two_sum(yl[0] - (float)P.black, -a);
                } else if (COMPOSITE) {
                    yb = two_sum(cb, -2.0f * __fmaf_rn(PY[s], carrier_sin(x), QY[s] * carrier_cos(x)));
                } else {
                    yb = two_sum(cb, -v[0][s + 7]);
                }
                const float U = -(PU[s] * bp + QU[s] * bq) * 2.0f;
                const float V = vsw * -(QV[s] * bp - PV[s] * bq) * 2.0f;
                if (vout) {
                    yuv_values(P, yb, U, V, o0[s], o1[s], o2[s]);
                } else if (x >= P.avs && x < P.ave) {
                    pack_sample(P, out_base, frame_slot, rowpix + (x - P.avs), yb, U, V);
                }
            }
        }
        if (!vout) continue;
        const float n0 = __shfl_down_sync(0xffffffffu, o0[0], 1);
        const float n1 = __shfl_down_sync(0xffffffffu, o1[0], 1);
        const float n2 = __shfl_down_sync(0xffffffffu, o2[0], 1);
        const int nitem = __shfl_down_sync(0xffffffffu, live ? item : -1, 1);
        const bool full = live && 8 * seg + 8 <= aw &&
                          (xoff == 0 || (lane < 31 && nitem == item + 1 && seg + 1 < per_line));
        const bool prev_full = (__shfl_up_sync(0xffffffffu, full ? 1 : 0, 1) != 0) && lane > 0;
        if (!live) continue;
        const long long e0 = frame_slot * P.out_frame_stride + rowpix;
        if (full) {
            float a0[8], a1[8], a2[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {   // xoff is 0 or 1 here; constant indices keep o* in registers
                a0[j] = xoff == 0 ? o0[j] : (j < 7 ? o0[j < 7 ? j + 1 : 7] : n0);
                a1[j] = xoff == 0 ? o1[j] : (j < 7 ? o1[j < 7 ? j + 1 : 7] : n1);
                a2[j] = xoff == 0 ? o2[j] : (j < 7 ? o2[j < 7 ? j + 1 : 7] : n2);
            }
            const long long e = e0 + 8 * seg;
            store8(P, out_base, e, a0);
            store8(P, out_base, e + plane, a1);
            store8(P, out_base, e + 2 * plane, a2);
        }
        // samples no vector store covered: edges, and sample 0 unless the
        // previous lane stored it
#pragma unroll
        for (int s = 0; s < 8; s++) {
            const int p = 8 * seg + s - xoff;
            if (p < 0 || p >= aw) continue;
            if (full && s >= xoff) continue;
            if (xoff == 1 && s == 0 && prev_full) continue;
            store_yuv(P, out_base, e0 + p, plane, o0[s], o1[s], o2[s]);
        }
    }
}

// PalColour::buildLookUpTables chroma taps (palcolour.cpp:197-276), in double,
// for the sample rate; -2 when the filter is longer than the kernel's 8 taps.
int demod_taps(double sample_rate, float (&cfilt)[8][4], float (&yfilt)[8][2])
{
    const double chromaBandwidthHz = 1100000.0 / 0.93;
    const double ca = 0.5 * sample_rate / chromaBandwidthHz;
    int fs = 1;
    if ((int)ca > fs) fs = (int)ca;
    if (fs > 7) return -2;
    double cf[8][4] = {}, yf[8][2] = {};
    double cdiv = 0, ydiv = 0;
    for (int f = 0; f <= fs; f++) {
        const double fc = std::min(ca, (double)f);
        const double ff = std::min(ca, sqrt((double)(f * f + 4)));
        const double fff = std::min(ca, sqrt((double)(f * f + 16)));
        const double ffff = std::min(ca, sqrt((double)(f * f + 36)));
        const int d = (f == 0) ? 2 : 1;
        cf[f][0] = (1 + cos(M_PI * fc / ca)) / d;
        cf[f][2] = (1 + cos(M_PI * ff / ca)) / d;
        cf[f][1] = (1 + cos(M_PI * fff / ca)) / d;
        cf[f][3] = (1 + cos(M_PI * ffff / ca)) / d;
        cdiv += 2 * (1 * cf[f][0] + 2 * cf[f][2] + 2 * cf[f][1] + 2 * cf[f][3]);
        // luma-extraction taps (ya = ca at this bandwidth)
        const double fy = std::min(ca, (double)f);
        const double fffy = std::min(ca, sqrt((double)(f * f + 16)));
        yf[f][0] = (1 + cos(M_PI * fy / ca)) / d;
        yf[f][1] = 0.2 * (1 + cos(M_PI * fffy / ca)) / d;
        ydiv += 2 * (1 * yf[f][0] + 2 * yf[f][1]);
    }
    for (int f = 0; f < 8; f++) {
        for (int i = 0; i < 4; i++) cfilt[f][i] = (float)(cf[f][i] / cdiv);
        for (int i = 0; i < 2; i++) yfilt[f][i] = (float)(yf[f][i] / ydiv);
    }
    return 0;
}

// The doYNR high-pass, once per device.
int demod_init_constants(int device)
{
    if (device >= 0 && device < 64 && g_demod_ready[device]) return 0;
    // c_nrpal_b, src/decoders/filter/deemp.h:620-628
    static const double nrpal[25] = {
        1.141291975113614e-04, -1.857019211291029e-03, -4.499636864042073e-03, -5.577680979937061e-03,
        -4.423694440267179e-04, 1.309163063177155e-02, 2.861211356202848e-02, 3.029931283148555e-02,
        1.098965697652802e-03, -6.398130386469833e-02, -1.492080690537196e-01, -2.223459379380252e-01,
        7.479077367478024e-01, -2.223459379380252e-01, -1.492080690537196e-01, -6.398130386469833e-02,
        1.098965697652803e-03, 3.029931283148557e-02, 2.861211356202848e-02, 1.309163063177156e-02,
        -4.423694440267185e-04, -5.577680979937061e-03, -4.499636864042074e-03, -1.857019211291030e-03,
        1.141291975113614e-04};
    float nrf[25];
    for (int i = 0; i < 25; i++) nrf[i] = (float)nrpal[i];
    if (cudaMemcpyToSymbol(cd_nrpal, nrf, sizeof(nrf)) != cudaSuccess) return -1;
    if (device >= 0 && device < 64) g_demod_ready[device] = true;
    return 0;
}

size_t demod_smem_bytes(int avs, int ave, bool ynr)
{
    const int span = demod_span(avs, ave);
    const int lines = demod_lines(ynr);
    const size_t rows = sizeof(float) * (size_t)(lines + 6) * (span + 2 * kPad);
    return rows + (ynr ? sizeof(float) * (size_t)lines * (span + 2 * kNrHalf) : 0);
}

int demod_launch(const DemodParams &P, cudaStream_t stream)
{
    if (P.nout <= 0) return 0;
    const bool composite = P.partial == nullptr;
    const bool ynr = P.nr_y > 0.f;
    const size_t smem = demod_smem_bytes(P.avs, P.ave, ynr);
    if (smem > 110 * 1024) return -1;   // two blocks per SM
    // function attributes are per device
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return -1;
    if (!attr_set[dev]) {
        const int lim = 110 * 1024;
        if (cudaFuncSetAttribute(demod_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
                cudaSuccess ||
            cudaFuncSetAttribute(demod_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
                cudaSuccess ||
            cudaFuncSetAttribute(demod_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
                cudaSuccess ||
            cudaFuncSetAttribute(demod_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
                cudaSuccess)
            return -1;
        attr_set[dev] = true;
    }
    const int lines = demod_lines(ynr);
    const int nblk_per_field = (P.fh + lines - 1) / lines;
    const dim3 grid((unsigned)(P.nout * nblk_per_field));
    if (composite) {
        if (ynr) demod_kernel<true, true><<<grid, kDemodThreads, smem, stream>>>(P);
        else demod_kernel<true, false><<<grid, kDemodThreads, smem, stream>>>(P);
    } else {
        if (ynr) demod_kernel<false, true><<<grid, kDemodThreads, smem, stream>>>(P);
        else demod_kernel<false, false><<<grid, kDemodThreads, smem, stream>>>(P);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace tpal
