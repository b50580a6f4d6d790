// tpal2d.cu -- Transform-PAL 2D chroma separation on sm_103a.
//
// Computes what the reference's TransformPal2D does
// (src/decoders/palcolour/transform_pal_2d.cpp:107-287): per field, 16-line x
// 32-sample raised-cosine-windowed tiles, half-overlapped, starting half a
// tile above/left of the active area; rows outside the field's active lines
// are black; forward real DFT; keep a bin and its mirror about the carrier
// (x_ref = 16 - x, y_ref = (8 - y) mod 16) when their squared magnitudes are
// within the threshold ratio, for x in [4, 8]; inverse DFT / 512 and
// overlap-add into the active window. GPU structure:
//
//  * one warp per tile: lanes (h, i) hold row i; half-warp h = 0 computes
//    bins kx 4..8, h = 1 bins 9..12 -- the only bins the filter can keep;
//  * black and each row's mean are subtracted first (they only touch bins
//    kx in {0, +-1} of the windowed row), so invalid rows are exact zeros;
//  * the 16-point Y DFT is a shuffle FFT across the half-warp;
//  * decisions are FP32 with a per-kx error bound; decisions inside it are
//    recomputed in double-float from the raw samples by the whole warp;
//  * overlap-add: tiles of one (tileY parity, tileX parity) class tile the
//    active area without overlap, so each class writes its own partial plane
//    (the same layout the 3D kernel writes, read by the demodulator).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "tpal_common.cuh"
#include "tpal_kernels.h"

namespace tpal {

__constant__ float c2_cwx[9][16];   // w32(x) cos(theta), theta = 2 pi kx (x - 15.5)/32, kx = 4..12, x < 16
__constant__ float c2_swx[9][16];   // w32(x) sin(theta)
__constant__ float c2_cix[9][16];   // (2/512) cos(theta)
__constant__ float c2_six[9][16];   // (2/512) sin(theta)
// the same as pairs for the f32x2 instructions: (cwx, -swx) and (cix, six)
__constant__ float2 c2_xf[9][16];
__constant__ float2 c2_xi[9][16];
__constant__ float c2_wx[16];       // w32(x), x < 16
__constant__ float c2_wy[16];       // w16(i)
__constant__ float2 c2_tw16[16];    // exp(-2 pi i r/16)
__constant__ float c2_dfx[9][32][4];  // w32(x) exp(-2 pi i kx x/32) as double-float re/im
__constant__ float c2_dfwy[16][2];
__constant__ float c2_dftw16[16][4];

static bool g_tp2_ready[64];

constexpr int kWarps2 = 4;
constexpr float kBound2 = 2.0f;
constexpr float kEps = 5.9604645e-8f;

__device__ __forceinline__ float2 cmul2(float2 a, float2 b)
{
    return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float2 shx(float2 v, int m)
{
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

__device__ __forceinline__ float l1f(float2 a) { return fabsf(a.x) + fabsf(a.y); }

struct Thr2 {
    float f;
    df d;
};

__device__ __forceinline__ Thr2 thr2(const T2Params &P, int frame, int ky, int kx)
{
    if (P.thr_table == nullptr) {
        if (P.frame_t2 != nullptr) {   // a batch of captures: the threshold of this frame's capture
            const float *t = P.frame_t2 + 3 * frame;
            return {t[0], {t[1], t[2]}};
        }
        return {P.t2f, {P.t2hi, P.t2lo}};
    }
    const float *t = P.thr_table + 3 * (ky * 5 + (kx - 4));
    return {t[0], {t[1], t[2]}};
}

// Exact (double-float) squared magnitudes of bin (kyb, kxb) and of its mirror.
__device__ __noinline__ void exact_pair2(const T2Params &P, int f, int tileX, int tileY, int fl_first, int fl_last,
                                         int kyb, int kxb, df &mb, df &mr)
{
    const int lane = threadIdx.x & 31;
    const int h = lane >> 4, i = lane & 15;
    const int ky = h ? ((8 - kyb) & 15) : kyb;
    const int kx = h ? 16 - kxb : kxb;
    const int fl = tileY + i;
    dfc acc = {{0.f, 0.f}, {0.f, 0.f}};
    const uint16_t *fp = field_at(P, f);   // f is an output field: inside the buffer or the table
    if (fp != nullptr && fl >= fl_first && fl < fl_last) {
        const uint16_t *row = fp + (long long)fl * P.fw;
        dfc x1 = acc;
        for (int x = 0; x < 32; x++) {
            const int xx = max(tileX + x, -fl * P.fw);
            const float a = (float)((int)row[xx] - P.black);
            const float *c = c2_dfx[kx - 4][x];
            x1.re = df_add(x1.re, df_mul_f({c[0], c[1]}, a));
            x1.im = df_add(x1.im, df_mul_f({c[2], c[3]}, a));
        }
        const int r = (ky * i) & 15;
        dfc w = {{c2_dftw16[r][0], c2_dftw16[r][1]}, {c2_dftw16[r][2], c2_dftw16[r][3]}};
        const df wy = {c2_dfwy[i][0], c2_dfwy[i][1]};
        w.re = df_mul(w.re, wy);
        w.im = df_mul(w.im, wy);
        acc = dfc_mul(x1, w);
    }
#pragma unroll
    for (int m = 1; m < 16; m <<= 1) acc = dfc_add(acc, dfc_shfl_xor(acc, m));
    const df mine = df_add(df_mul(acc.re, acc.re), df_mul(acc.im, acc.im));
    const df other = df_shfl_xor(mine, 16);
    mb = h ? other : mine;
    mr = h ? mine : other;
}

__device__ __forceinline__ bool sim2(float a, float b, float t)
{
    return (__fmaf_rn(-b, t, a) >= 0.f) && (__fmaf_rn(-a, t, b) >= 0.f);
}

__device__ __forceinline__ bool unc2(float a, float b, float t, float pa, float pb)
{
    // Two bins that are exactly zero with a zero error bound (a flat or
    // black tile) need no exact pass: both outputs are zero either way.
    return ((fabsf(__fmaf_rn(-b, t, a)) <= pa + t * pb) || (fabsf(__fmaf_rn(-a, t, b)) <= pb + t * pa)) &&
           (a + b + pa + pb > 0.f);
}

__device__ __forceinline__ bool df_sim2(df a, df b, df t)
{
    const df d1 = df_sub(a, df_mul(b, t));
    const df d2 = df_sub(b, df_mul(a, t));
    return !(df_sign(d1) < 0 || df_sign(d2) < 0);
}

template <bool PER_BIN>
__global__ void __launch_bounds__(32 * kWarps2) tpal2d_kernel(T2Params P)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int h = lane >> 4, i = lane & 15;
    const int tileX0 = P.avs - 16;
    const int ntx = (P.ave - tileX0 + 15) / 16;
    // tile rows: the larger of the two field parities' grids
    const int nty = max((((P.lafl - 0) / 2 + 1) - ((P.fafl + 1 - 0) / 2 - 8) + 7) / 8,
                        (((P.lafl - 1) / 2 + 1) - ((P.fafl + 1 - 1) / 2 - 8) + 7) / 8);
    const long long item = (long long)blockIdx.x * kWarps2 + warp;
    const long long per_field = (long long)ntx * nty;
    if (item >= per_field * P.nout) return;
    const int o = (int)(item / per_field);
    const int t = (int)(item % per_field);
    const int tx = t % ntx, ty = t / ntx;
    const int f = P.field_begin + o;
    const int off = (f & 1) ^ P.swap;   // SourceField::getOffset
    const int fl_first = (P.fafl + 1 - off) / 2;   // SourceField::getFirstActiveLine
    const int fl_last = ((P.lafl - off) / 2) + 1;  // SourceField::getLastActiveLine
    const int tileY = fl_first - 8 + 8 * ty;
    if (tileY >= fl_last) return;
    const int tileX = tileX0 + 16 * tx;
    const int cls = ((ty & 1) << 1) | (tx & 1);
    const int nk = h ? 4 : 5;     // bins kx 4..8 (h = 0) or 9..12 (h = 1)
    const int kbase = h ? 5 : 0;  // index into the kx = 4..12 tables

    // --- forward X: row i, DC/black removed, folded about the window centre
    const int fl = tileY + i;
    const uint16_t *fp = (f >= 0 && f < P.nfields) ? field_at(P, f) : nullptr;
    const bool valid = (fp != nullptr) && (fl >= fl_first) && (fl < fl_last);
    float2 sd[16];   // (s_x, d_x)
    float rowl1 = 0.f;
    if (valid) {
        const uint16_t *row = fp + (long long)fl * P.fw;
        int a[32];
        int sum = 0;
#pragma unroll
        for (int x = 0; x < 32; x++) {
            const int xx = max(tileX + x, -fl * P.fw);
            a[x] = (int)__ldg(row + xx) - P.black;
            sum += a[x];
        }
        const float m32 = (float)sum * 0.03125f;
#pragma unroll
        for (int x = 0; x < 16; x++) {
            sd[x] = make_float2((float)(16 * (a[x] + a[31 - x]) - sum) * 0.0625f,   // a_x + a_31-x - 2 mean (exact)
                                (float)(a[x] - a[31 - x]));
            rowl1 = __fmaf_rn(c2_wx[x], fabsf((float)a[x] - m32) + fabsf((float)a[31 - x] - m32), rowl1);
        }
    } else {
#pragma unroll
        for (int x = 0; x < 16; x++) sd[x] = make_float2(0.f, 0.f);
    }
    const float wy = c2_wy[i];
    rowl1 *= wy;
#pragma unroll
    for (int m = 1; m < 16; m <<= 1) rowl1 += __shfl_xor_sync(0xffffffffu, rowl1, m);

    // per-lane FFT twiddles (DIF stages h = 8, 4, 2, 1)
    float2 tw[4];
    {
        int s = 0;
#pragma unroll
        for (int hh = 8; hh >= 1; hh >>= 1, s++) tw[s] = c2_tw16[(i & (hh - 1)) * (8 / hh)];
    }

    float2 Y[5];
    float E[5];
    // Every lane runs all five bins (the shuffles below need the whole
    // warp); half-warp 1 has only four, its fifth is a zero dummy.
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const bool real = k < nk;
        const int row = real ? kbase + k : 8;
        float2 X = make_float2(0.f, 0.f);
#pragma unroll
        for (int x = 0; x < 16; x++) {
            X = __ffma2_rn(c2_xf[row][x], sd[x], X);   // (cwx sx + .., -swx dx + ..)
        }
        const float wk = real ? wy : 0.f;
        X.x *= wk;
        X.y *= wk;
        float A = l1f(X);
#pragma unroll
        for (int m = 1; m < 16; m <<= 1) A += __shfl_xor_sync(0xffffffffu, A, m);
        E[k] = kBound2 * kEps * (A + 0.5f * rowl1);
        // 16-point DFT over rows (DIF; lane i ends with bin rev4(i))
        int s = 0;
#pragma unroll
        for (int hh = 8; hh >= 1; hh >>= 1, s++) {
            const bool upper = (i & hh) != 0;
            const float2 ov = shx(X, hh);
            X = upper ? cmul2(sub2(ov, X), tw[s]) : add2(X, ov);
        }
        Y[k] = X;
    }
    const int ky = rev4(i);
    const int kyr = (8 - ky) & 15;
    // half-0 lane (ky) pairs with half-1 lane rev4(kyr) for kx 4..7, and with
    // half-0 lane rev4(kyr) for kx 8.
    const int mirror_other = 16 + rev4(kyr);
    const int mirror_same = rev4(kyr);
    float mag[5], ab[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        mag[k] = __fmaf_rn(Y[k].x, Y[k].x, Y[k].y * Y[k].y);
        ab[k] = l1f(Y[k]);
    }
    // Mirror data: for my bin kx (h = 0, k < 4) the mirror is kx' = 16 - kx,
    // index k' = 3 - k in half 1; for kx = 8 (k = 4) it is k = 4 in half 0.
    float rm[5], ra[5], rE[5];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int src = (h == 0) ? mirror_other : 0;
        rm[k] = __shfl_sync(0xffffffffu, mag[3 - k], src);
        ra[k] = __shfl_sync(0xffffffffu, ab[3 - k], src);
        rE[k] = __shfl_sync(0xffffffffu, E[3 - k], src);
    }
    rm[4] = __shfl_sync(0xffffffffu, mag[4], mirror_same);
    ra[4] = __shfl_sync(0xffffffffu, ab[4], mirror_same);
    rE[4] = __shfl_sync(0xffffffffu, E[4], mirror_same);

    unsigned keep = 0, unc = 0;
    if (h == 0) {
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const int kx = 4 + k;
            const bool self = (kx == 8) && (ky == kyr);
            const float a = mag[k], b = rm[k];
            const float pa = 2.f * E[k] * ab[k] + E[k] * E[k];
            const float pb = 2.f * rE[k] * ra[k] + rE[k] * rE[k];
            float tt = (P.frame_t2 != nullptr) ? P.frame_t2[3 * (f >> 1)] : P.t2f;
            if (PER_BIN) tt = thr2(P, f >> 1, ky, kx).f;
            bool sm = sim2(a, b, tt);
            bool u = unc2(a, b, tt, pa, pb);
            if (PER_BIN && kx == 8) {   // the mirror (also kx 8) visits with its own threshold
                const float t2 = thr2(P, f >> 1, kyr, 8).f;
                sm |= sim2(a, b, t2);
                u |= unc2(a, b, t2, pa, pb);
            }
            if (sm || self) keep |= 1u << k;
            if (u && !self) unc |= 1u << k;
        }
    }
    unsigned n_exact = 0, n_flip = 0;
    unsigned any = __ballot_sync(0xffffffffu, unc != 0);
    while (any) {
        const int src = __ffs(any) - 1;
        const unsigned su = __shfl_sync(0xffffffffu, unc, src);
        const int k = __ffs(su) - 1;
        const int kyb = rev4(src & 15), kxb = 4 + k;
        df mb, mr;
        exact_pair2(P, f, tileX, tileY, fl_first, fl_last, kyb, kxb, mb, mr);
        const int kybr = (8 - kyb) & 15;
        bool sm = df_sim2(mb, mr, thr2(P, f >> 1, kyb, kxb).d);
        if (kxb == 8) sm |= df_sim2(mb, mr, thr2(P, f >> 1, kybr, 8).d);
        if (lane == src) {
            n_exact++;
            if ((((keep >> k) & 1u) != 0) != sm) n_flip++;
            keep = sm ? (keep | (1u << k)) : (keep & ~(1u << k));
            unc &= ~(1u << k);
        }
        if (kxb == 8 && lane == rev4(kybr)) {   // the kx-8 mirror is a visitor too
            keep = sm ? (keep | (1u << 4)) : (keep & ~(1u << 4));
            unc &= ~(1u << 4);
        }
        any = __ballot_sync(0xffffffffu, unc != 0);
    }
    // Half 1 bins (kx 9..12, index k) are kept when their mirror (kx 16-kx,
    // index 3-k, on half-0 lane rev4(kyr)) was kept.
    {
        const unsigned mk = __shfl_sync(0xffffffffu, keep, rev4(kyr));
        if (h == 1) {
            keep = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) keep |= ((mk >> (3 - k)) & 1u) << k;
        }
    }

    // --- inverse Y (DIT, bit-reversed in -> natural rows out) and X partial sums
    float2 CS[16];   // (cosine sum, sine sum)
#pragma unroll
    for (int x = 0; x < 16; x++) CS[x] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 5; k++) {   // all lanes, all five bins (shuffles); half 1's fifth is zero
        const int row = (k < nk) ? kbase + k : 8;
        float2 G = (((keep >> k) & 1u) && k < nk) ? Y[k] : make_float2(0.f, 0.f);
        int s = 3;
#pragma unroll
        for (int hh = 1; hh <= 8; hh <<= 1, s--) {
            const bool upper = (i & hh) != 0;
            const float2 w = make_float2(tw[s].x, -tw[s].y);
            const float2 ov = shx(G, hh);
            const float2 tt = cmul2(upper ? G : ov, w);
            G = upper ? sub2(ov, tt) : add2(G, tt);
        }
#pragma unroll
        for (int x = 0; x < 16; x++) CS[x] = __ffma2_rn(G, c2_xi[row][x], CS[x]);
    }
#pragma unroll
    for (int x = 0; x < 16; x++) CS[x] = add2(CS[x], shx(CS[x], 16));
    if (fl >= fl_first && fl < fl_last) {
        float *dst = P.partial + (long long)cls * P.part_class_stride + (long long)o * P.part_field_stride +
                     (long long)(fl - P.fl_lo) * P.part_row_stride - P.avs;
        // this lane's 16 samples [tileX + 16 h, +16): tileX - avs is a multiple
        // of 16, so inside the active window they start on a 64-byte boundary
        // whenever the planes' strides are multiples of 4 floats and their
        // base is 16-byte aligned: four vector stores
        const int x0 = tileX + 16 * h;
        const bool vec = ((P.part_row_stride | P.part_field_stride | P.part_class_stride) & 3) == 0 &&
                         (reinterpret_cast<uintptr_t>(P.partial) & 15) == 0 && x0 >= P.avs && x0 + 16 <= P.ave;
        if (vec) {
            float v[16];
#pragma unroll
            for (int x = 0; x < 16; x++) {
                if (h) v[15 - x] = CS[x].x + CS[x].y;
                else v[x] = CS[x].x - CS[x].y;
            }
            float4 *d4 = reinterpret_cast<float4 *>(dst + x0);
#pragma unroll
            for (int q = 0; q < 4; q++) d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else {
#pragma unroll
            for (int x = 0; x < 16; x++) {
                const int X = h ? tileX + 31 - x : tileX + x;
                if (X >= P.avs && X < P.ave) dst[X] = h ? CS[x].x + CS[x].y : CS[x].x - CS[x].y;
            }
        }
    }
    if (P.stats != nullptr) {
        if (n_exact) atomicAdd(P.stats + 0, n_exact);
        if (n_flip) atomicAdd(P.stats + 1, n_flip);
    }
}

static double rc_window2(int n, int N) { return 0.5 - (0.5 * cos((2 * M_PI * (n + 0.5)) / N)); }

static void split2(double v, float &hi, float &lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

int tp2_init_constants(int device)
{
    if (device >= 0 && device < 64 && g_tp2_ready[device]) return 0;
    float cwx[9][16], swx[9][16], cix[9][16], six[9][16], wx[16], wy[16];
    for (int k = 0; k < 9; k++) {
        const int kx = 4 + k;
        for (int x = 0; x < 16; x++) {
            const double th = 2.0 * M_PI * kx * (x - 15.5) / 32.0;
            const double w = rc_window2(x, 32);
            cwx[k][x] = (float)(w * cos(th));
            swx[k][x] = (float)(w * sin(th));
            cix[k][x] = (float)((2.0 / 512.0) * cos(th));
            six[k][x] = (float)((2.0 / 512.0) * sin(th));
        }
    }
    for (int x = 0; x < 16; x++) wx[x] = (float)rc_window2(x, 32);
    for (int i = 0; i < 16; i++) wy[i] = (float)rc_window2(i, 16);
    float2 tw[16];
    for (int r = 0; r < 16; r++) tw[r] = make_float2((float)cos(-2 * M_PI * r / 16), (float)sin(-2 * M_PI * r / 16));
    float dfx[9][32][4], dfwy[16][2], dftw[16][4];
    for (int k = 0; k < 9; k++)
        for (int x = 0; x < 32; x++) {
            const double w = rc_window2(x, 32), a = -2.0 * M_PI * (4 + k) * x / 32.0;
            split2(w * cos(a), dfx[k][x][0], dfx[k][x][1]);
            split2(w * sin(a), dfx[k][x][2], dfx[k][x][3]);
        }
    for (int i = 0; i < 16; i++) split2(rc_window2(i, 16), dfwy[i][0], dfwy[i][1]);
    for (int r = 0; r < 16; r++) {
        split2(cos(-2 * M_PI * r / 16), dftw[r][0], dftw[r][1]);
        split2(sin(-2 * M_PI * r / 16), dftw[r][2], dftw[r][3]);
    }
#define TP2_CPY(sym, src) \
    if (cudaMemcpyToSymbol(sym, src, sizeof(src)) != cudaSuccess) return -1;
    TP2_CPY(c2_cwx, cwx);
    TP2_CPY(c2_swx, swx);
    TP2_CPY(c2_cix, cix);
    TP2_CPY(c2_six, six);
    float2 xf[9][16], xi[9][16];
    for (int k = 0; k < 9; k++)
        for (int x = 0; x < 16; x++) {
            xf[k][x] = make_float2(cwx[k][x], -swx[k][x]);
            xi[k][x] = make_float2(cix[k][x], six[k][x]);
        }
    TP2_CPY(c2_xf, xf);
    TP2_CPY(c2_xi, xi);
    TP2_CPY(c2_wx, wx);
    TP2_CPY(c2_wy, wy);
    TP2_CPY(c2_tw16, tw);
    TP2_CPY(c2_dfx, dfx);
    TP2_CPY(c2_dfwy, dfwy);
    TP2_CPY(c2_dftw16, dftw);
#undef TP2_CPY
    if (device >= 0 && device < 64) g_tp2_ready[device] = true;
    return 0;
}

int tp2_launch(const T2Params &P, cudaStream_t stream)
{
    const int tileX0 = P.avs - 16;
    const int ntx = (P.ave - tileX0 + 15) / 16;
    const int nty = std::max((((P.lafl - 0) / 2 + 1) - ((P.fafl + 1 - 0) / 2 - 8) + 7) / 8,
                             (((P.lafl - 1) / 2 + 1) - ((P.fafl + 1 - 1) / 2 - 8) + 7) / 8);
    const long long items = (long long)ntx * nty * P.nout;
    if (items <= 0) return 0;
    const unsigned blocks = (unsigned)((items + kWarps2 - 1) / kWarps2);
    if (P.thr_table != nullptr) tpal2d_kernel<true><<<blocks, 32 * kWarps2, 0, stream>>>(P);
    else tpal2d_kernel<false><<<blocks, 32 * kWarps2, 0, stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace tpal
