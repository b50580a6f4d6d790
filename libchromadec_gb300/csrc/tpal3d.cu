// tpal3d.cu -- Transform-PAL 3D chroma separation on sm_103a.
//
// Computes exactly what the reference's TransformPal3D does
// (src/decoders/palcolour/transform_pal_3d.cpp:123-333): 8x32x16 (fields x
// frame lines x samples) raised-cosine-windowed tiles, half-overlapped, with
// the Z tiles anchored per frame (tiles start at fields 2k-4 and 2k for frame
// k), a forward real DFT, the mirror-about-the-subcarrier threshold, the
// inverse DFT and overlap-add -- restructured for the GPU:
//
//  * One warp owns one spatial tile position (tileX, tileY) and walks forward
//    through a chunk of frames. The 3D DFT is separable, and the X (samples)
//    and Y (frame lines) stages of a field do not depend on which Z tile the
//    field sits in, so each field's 2D spectrum S_f[ky][kx] is computed once
//    and reused by the four Z tiles that contain it. Only kx = 2..6 is ever
//    needed: the filter reads and writes bins x in [XTILE/8, XTILE/4] and
//    their mirrors 8-x (transform_pal_3d.cpp:294-331), so every other bin of
//    the inverse is zero.
//  * Rows of the other field's parity are black (transform_pal_3d.cpp:185-190).
//    Subtracting black (and each row's own mean) before the DFT changes only
//    bins kx in {0, +-1} because the raised cosine's spectrum is supported on
//    {0, +-1}; so those rows become exact zeros and the 32-point Y DFT of a
//    field is a 16-point DFT of its own-parity rows plus a parity twiddle.
//  * Output field 2k gets slice 0 of tile 2k and slice 4 of tile 2k-4
//    (transform_pal_3d.cpp:214-215); the two are summed in the spectral domain
//    and one inverse Y/X transform runs per output field.
//  * Overlap-add across spatial tiles: tiles of one (tileY parity, tileX
//    parity) class never overlap and cover the active area, so each class
//    writes its own partial plane and the demodulator sums the four planes.
//    No atomics; results are deterministic.
//  * Threshold decisions: the spectrum is computed in FP32 with a per-bin
//    error bound E = K * 2^-24 * (sum_z w_z (A_z[kx] + R_z/2) + sum_z w_z |S_z|_1)
//    where A is the L1 norm of the field's column-DFT outputs for that kx and R
//    the L1 norm of its DC-removed windowed rows. A decision whose margin is
//    inside the bound is recomputed by the whole warp in double-float from the
//    raw samples, so every decision equals the FP64 reference's.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "tpal_common.cuh"
#include "tpal_kernels.h"

namespace tpal {

// ---------------------------------------------------------------------------
// Constant tables (filled by tp3_init_constants from double precision)
// ---------------------------------------------------------------------------
// X-stage tables as (re, im) pairs for the paired FP32 instructions
// (fma.rn.f32x2: two independent round-to-nearest FMAs, the same results as
// two scalar FMAs, in one instruction):
__constant__ float2 c3_xf[5][8];   // forward X: w(x) (cos theta_kx, -sin theta_kx), theta = 2 pi kx (x - 7.5) / 16
__constant__ float2 c3_xi[5][8];   // inverse X: (2/4096) (cos theta, sin theta)
__constant__ float c3_wy[2][16];   // w_y(y0 + 2i), 32-point raised cosine
__constant__ float c3_wx[16];      // w_x(x)
__constant__ float c3_wz[8];       // w_z(z)
__constant__ float2 c3_tw16[16];   // exp(-2 pi i r / 16)
__constant__ float2 c3_tw32[32];   // exp(-2 pi i r / 32)
// double-float tables for the exact decision path
// w_x(x) exp(-2 pi i kx x/16) as 60-bit fixed point, c * 2^60 = hi * 2^30 + lo
// (lo in [0, 2^30)): re.hi, re.lo, im.hi, im.lo
__constant__ int c3_qx[5][16][4];
__constant__ float c3_dfwy[32][2];     // w_y(y)
__constant__ float c3_dfwz[8][2];      // w_z(z)
__constant__ float c3_dftw32[32][4];   // exp(-2 pi i r/32)

static bool g_tp3_constants_ready[64];

// kappa(lane): the ky a lane owns in the Z stage (bit-reversed low nibble, so
// it matches the order the shuffle FFT leaves the spectrum in); an involution.
__device__ __forceinline__ int kappa(int l) { return rev4(l & 15) | (l & 16); }

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float l1(float2 a) { return fabsf(a.x) + fabsf(a.y); }

// multiply by -i: (y, -x); by the tables' exp(-i pi/2) = (6e-17, -1), whose
// tiny real part is below the rounding of any non-degenerate product
__device__ __forceinline__ float2 mul_negi(float2 a) { return make_float2(a.y, -a.x); }

__device__ __forceinline__ float2 shfl_xor2(float2 v, int m)
{
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

__device__ __forceinline__ float2 shfl2(float2 v, int src)
{
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

__device__ __forceinline__ df dfc_abs2(dfc v) { return df_add(df_mul(v.re, v.re), df_mul(v.im, v.im)); }

__device__ __forceinline__ dfc dfc_tw32(int r)
{
    r &= 31;
    return {{c3_dftw32[r][0], c3_dftw32[r][1]}, {c3_dftw32[r][2], c3_dftw32[r][3]}};
}

// Squared threshold of visited bin (z, y, x-2) for x in 2..4.
struct Thr {
    float f;
    df d;
};

__device__ __forceinline__ Thr thr_of(const T3Params &P, int m, int kz, int ky, int kx)
{
    if (P.thr_table == nullptr) {
        if (P.frame_t2 != nullptr) {   // a batch of captures: the threshold of frame m's capture
            const float *t = P.frame_t2 + 3 * max(m, 0);   // warm-up steps before frame 0 take frame 0's
            return {t[0], {t[1], t[2]}};
        }
        return {P.t2f, {P.t2hi, P.t2lo}};
    }
    const float *t = P.thr_table + 3 * ((kz * 32 + ky) * 3 + (kx - 2));
    return {t[0], {t[1], t[2]}};
}

// ---------------------------------------------------------------------------
// Per-lane constants of the forward/inverse stages (fixed for the whole walk:
// lane (j, i) always handles row i of the field with offset j).
// ---------------------------------------------------------------------------
struct LaneConst {
    int j, i, y0, kk;
    float wy;          // w_y(y0 + 2i)
    float2 ftw[4];     // radix-2 stage twiddles, h = 8, 4, 2, 1: exp(-2 pi i r / 2h)
    float2 ptw;        // exp(-2 pi i kk y0 / 32)
};

__device__ __forceinline__ LaneConst lane_const(int lane, int tileY, int swap)
{
    LaneConst c;
    c.j = lane >> 4;
    c.i = lane & 15;
    c.y0 = ((c.j ^ swap) - tileY) & 1;   // field offset (j ^ swap): its rows have that parity
    c.kk = rev4(c.i);
    c.wy = c3_wy[c.y0][c.i];
    int s = 0;
#pragma unroll
    for (int h = 8; h >= 1; h >>= 1, s++) c.ftw[s] = c3_tw16[(c.i & (h - 1)) * (8 / h)];
    c.ptw = c.y0 ? c3_tw32[c.kk] : make_float2(1.f, 0.f);
    return c;
}

// ---------------------------------------------------------------------------
// Forward X and Y stages of fields 2q (half-warp 0) and 2q+1 (half-warp 1).
// Writes S_f[kappa(l)][kx] into the shared window slot f & 7 and the bound
// terms of both fields into bnd[f & 7].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void forward_pair(const T3Params &P, int q, int tileX, int tileY, const LaneConst &LC,
                                             int lane, float2 *win /* [8][5][32] */, float *bnd /* [8][8] */)
{
    const int f = 2 * q + LC.j;
    const int L = tileY + LC.y0 + 2 * LC.i;   // frame line of this lane's row
    const uint16_t *fp = (f >= 0 && f < P.nfields) ? field_at(P, f) : nullptr;
    const bool valid = (fp != nullptr) && (L >= P.fafl) && (L <= P.lafl);

    // Row samples with black and the row mean removed, folded about the
    // window's centre: s_x = a_x + a_15-x - 2*mean, d_x = a_x - a_15-x
    // (exact in FP32); the window weight wy is applied to both.
    float2 sd[8];   // (s_x, d_x)
    float rowl1 = 0.0f;
    if (valid) {
        const uint16_t *row = fp + (long long)(L >> 1) * P.fw;
        int a[16];
        int sum = 0;
        if (tileX >= 0 && (L >> 1) >= 1 && ((L >> 1) + 1 < P.fh || tileX + 18 <= P.fw)) {
            // Rows start on any 2-byte boundary (odd line and field
            // lengths): nine aligned 32-bit words cover the 16 samples, and a
            // funnel shift by 0 or 16 bits lines each pair up -- 9 loads
            // instead of 16, each warp load touching 32 rows either way. The
            // words span at most the sample before and two after the 16,
            // inside the field: the row is not its first, and it is not the
            // last unless the words end inside it.
            const uintptr_t pa = reinterpret_cast<uintptr_t>(row + tileX);
            const uint32_t *w = reinterpret_cast<const uint32_t *>(pa & ~(uintptr_t)3);
            const unsigned sh = (unsigned)(pa & 2) * 8u;
            uint32_t wd[9];
#pragma unroll
            for (int k = 0; k < 9; k++) wd[k] = __ldg(w + k);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t v = __funnelshift_r(wd[k], wd[k + 1], sh);
                a[2 * k] = (int)(v & 0xFFFFu) - P.black;
                a[2 * k + 1] = (int)(v >> 16) - P.black;
            }
#pragma unroll
            for (int x = 0; x < 16; x++) sum += a[x];
        } else {
#pragma unroll
            for (int x = 0; x < 16; x++) {
                const int xx = max(tileX + x, -(L >> 1) * P.fw);   // never before the field start
                a[x] = (int)__ldg(row + xx) - P.black;
                sum += a[x];
            }
        }
        const float m16 = (float)sum * 0.0625f;
#pragma unroll
        for (int x = 0; x < 8; x++) {
            sd[x] = make_float2((float)(8 * (a[x] + a[15 - x]) - sum) * 0.125f, (float)(a[x] - a[15 - x]));
            rowl1 = __fmaf_rn(c3_wx[x], fabsf((float)a[x] - m16) + fabsf((float)a[15 - x] - m16), rowl1);
        }
    } else {
#pragma unroll
        for (int x = 0; x < 8; x++) sd[x] = make_float2(0.f, 0.f);
    }
    rowl1 *= LC.wy;
#pragma unroll
    for (int h = 1; h < 16; h <<= 1) rowl1 += __shfl_xor_sync(0xffffffffu, rowl1, h);
    const int fslot = f & 7;
    if (LC.i == 0) bnd[8 * fslot + 5] = rowl1;
    const int f0slot = (2 * q) & 7;

#pragma unroll
    for (int k = 0; k < 5; k++) {
        // column DFT bin kx = k+2 of this row (window and centre phase folded)
        float2 X = make_float2(0.f, 0.f);
#pragma unroll
        for (int x = 0; x < 8; x++) X = __ffma2_rn(c3_xf[k][x], sd[x], X);
        X = __fmul2_rn(X, make_float2(LC.wy, LC.wy));
        // bound term: sum over the field's rows of |X|_1
        float A = l1(X);
#pragma unroll
        for (int h = 1; h < 16; h <<= 1) A += __shfl_xor_sync(0xffffffffu, A, h);
        if (LC.i == 0) bnd[8 * fslot + k] = A;
        // 16-point DFT over the half-warp's rows (radix-2 DIF; lane i ends
        // with bin rev4(i))
        int st = 0;
#pragma unroll
        for (int h = 8; h >= 1; h >>= 1, st++) {
            const bool upper = (LC.i & h) != 0;
            const float2 o = shfl_xor2(X, h);
            X = upper ? cmul(sub2(o, X), LC.ftw[st]) : add2(X, o);
        }
        // parity twiddle: S[kk] = exp(-2 pi i kk y0/32) A[kk], S[kk+16] = (-1)^y0 S[kk];
        // swap halves so lane l holds both fields at ky = kappa(l)
        const float2 lo = cmul(X, LC.ptw);
        const float2 hi = LC.y0 ? make_float2(-lo.x, -lo.y) : lo;
        const float2 recv = shfl_xor2(LC.j ? lo : hi, 16);
        win[(f0slot * 5 + k) * 32 + lane] = LC.j ? recv : lo;            // field 2q
        win[((f0slot + 1) * 5 + k) * 32 + lane] = LC.j ? hi : recv;      // field 2q+1
    }
}

// ---------------------------------------------------------------------------
// Double-float X stage of one row for columns kx and 8 - kx. The second
// column's coefficients are the first's conjugated with sign (-1)^x
// (w(x) exp(-2 pi i (8-k) x / 16) = (-1)^x conj(w(x) exp(-2 pi i k x / 16))),
// so the products are formed once and summed twice.
// ---------------------------------------------------------------------------
// An integer below 2^51 in magnitude as double-float, through 32-bit
// conversions (the 64-bit ones run on the FP64 pipe, which this GPU has
// little of): v = hi * 2^32 + mid * 2^16 + low, each part exact in FP32.
__device__ __forceinline__ df df_from_i51(long long v)
{
    const float fh = (float)(int)(v >> 32) * 4294967296.0f;   // |v >> 32| < 2^19: exact
    const unsigned lo = (unsigned)v;
    const float fm = (float)(lo >> 16) * 65536.0f, fl = (float)(lo & 0xFFFFu);
    return df_add(two_sum(fh, fm), df_make(fl));
}

__device__ __forceinline__ df df_from_fixed60(long long hi_acc, long long lo_acc)
{
    // v = hi_acc * 2^-30 + lo_acc * 2^-60; hi_acc and lo_acc are below 2^51
    const df v = df_add(df_from_i51(hi_acc), df_make((float)(int)(lo_acc >> 30) + (float)(int)(lo_acc & 0x3FFFFFFF) *
                                                                                    9.3132257461547852e-10f));
    return {v.hi * 9.3132257461547852e-10f, v.lo * 9.3132257461547852e-10f};   // 2^-30
}

// The X stage in 60-bit fixed point: each sample times each coefficient
// word is an exact 64-bit integer product, so the sums are exact and the one
// rounding is the conversion to double-float (about 2^-47 of the sum).
__device__ __forceinline__ void x_row_pair(const uint16_t *field, long long base, long long field_len, int black,
                                           int kx, dfc &xa, dfc &xb)
{
    // even and odd samples summed apart: column kx is even + odd, column
    // 8 - kx ((-1)^x times the conjugate) is the conjugate of even - odd --
    // the same integers as summing each column's products directly
    long long e[4] = {0, 0, 0, 0}, o[4] = {0, 0, 0, 0};   // re.hi, re.lo, im.hi, im.lo
    int a[16];
    if (base >= 1 && base + 18 <= field_len) {
        // nine aligned 32-bit words and a funnel shift, as in forward_pair
        const uintptr_t pa = reinterpret_cast<uintptr_t>(field + base);
        const uint32_t *w = reinterpret_cast<const uint32_t *>(pa & ~(uintptr_t)3);
        const unsigned sh = (unsigned)(pa & 2) * 8u;
        uint32_t wd[9];
#pragma unroll
        for (int k = 0; k < 9; k++) wd[k] = __ldg(w + k);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t v = __funnelshift_r(wd[k], wd[k + 1], sh);
            a[2 * k] = (int)(v & 0xFFFFu) - black;
            a[2 * k + 1] = (int)(v >> 16) - black;
        }
    } else {
#pragma unroll
        for (int x = 0; x < 16; x++) {
            const long long idx = base + x < 0 ? 0 : base + x;   // never before the field start
            a[x] = (int)__ldg(field + idx) - black;
        }
    }
#pragma unroll
    for (int x = 0; x < 16; x++) {
        const int *c = c3_qx[kx - 2][x];
        long long *acc = (x & 1) ? o : e;
#pragma unroll
        for (int k = 0; k < 4; k++) acc[k] += (long long)a[x] * c[k];
    }
    xa = {df_from_fixed60(e[0] + o[0], e[1] + o[1]), df_from_fixed60(e[2] + o[2], e[3] + o[3])};
    xb = {df_from_fixed60(e[0] - o[0], e[1] - o[1]), df_from_fixed60(o[2] - e[2], o[3] - e[3])};
}

// ---------------------------------------------------------------------------
// Exact (double-float) magnitudes of bin b = (kzb, kyb, kxb) and its mirror
// r of Z tile T(2m). All 32 lanes cooperate; every lane returns the result.
// ---------------------------------------------------------------------------
__device__ __noinline__ void exact_pair(const T3Params &P, int m, int tileX, int tileY, int kzb, int kyb, int kxb,
                                        df &mb, df &mr)
{
    const int lane = threadIdx.x & 31;
    const int kzr = (10 - kzb) & 7, kyr = (40 - kyb) & 31;
    const int z = lane >> 2;
    const int part = lane & 3;
    const int f = 2 * m + z;
    const int p = (f & 1) ^ P.swap;   // SourceField::getOffset of window field f
    const int y0 = (p - tileY) & 1;
    dfc accb = {{0.f, 0.f}, {0.f, 0.f}}, accr = accb;
    const uint16_t *fp = (f >= 0 && f < P.nfields) ? field_at(P, f) : nullptr;
    if (fp != nullptr) {
        for (int r4 = 0; r4 < 4; r4++) {
            const int i = part * 4 + r4;
            const int y = y0 + 2 * i;
            const int L = tileY + y;
            if (L < P.fafl || L > P.lafl) continue;
            const long long base = (long long)(L >> 1) * P.fw + tileX;   // within the field
            dfc xb, xr;
            x_row_pair(fp, base, (long long)P.fh * P.fw, P.black, kxb, xb, xr);
            const df wy = {c3_dfwy[y][0], c3_dfwy[y][1]};
            dfc cb = dfc_tw32(kyb * y), cr = dfc_tw32(kyr * y);
            cb.re = df_mul(cb.re, wy); cb.im = df_mul(cb.im, wy);
            cr.re = df_mul(cr.re, wy); cr.im = df_mul(cr.im, wy);
            accb = dfc_add(accb, dfc_mul(xb, cb));
            accr = dfc_add(accr, dfc_mul(xr, cr));
        }
    }
    accb = dfc_add(accb, dfc_shfl_xor(accb, 1));
    accb = dfc_add(accb, dfc_shfl_xor(accb, 2));
    accr = dfc_add(accr, dfc_shfl_xor(accr, 1));
    accr = dfc_add(accr, dfc_shfl_xor(accr, 2));
    {
        const df wz = {c3_dfwz[z][0], c3_dfwz[z][1]};
        dfc tb = dfc_tw32(4 * ((kzb * z) & 7)), tr = dfc_tw32(4 * ((kzr * z) & 7));
        tb.re = df_mul(tb.re, wz); tb.im = df_mul(tb.im, wz);
        tr.re = df_mul(tr.re, wz); tr.im = df_mul(tr.im, wz);
        accb = dfc_mul(accb, tb);
        accr = dfc_mul(accr, tr);
    }
    // sum the 8 fields (lanes differing in bits 2..4; the 4 lanes of a field
    // hold identical values, so only lane bits 2..4 are combined)
    accb = dfc_add(accb, dfc_shfl_xor(accb, 4));
    accb = dfc_add(accb, dfc_shfl_xor(accb, 8));
    accb = dfc_add(accb, dfc_shfl_xor(accb, 16));
    accr = dfc_add(accr, dfc_shfl_xor(accr, 4));
    accr = dfc_add(accr, dfc_shfl_xor(accr, 8));
    accr = dfc_add(accr, dfc_shfl_xor(accr, 16));
    mb = dfc_abs2(accb);
    mr = dfc_abs2(accr);
}

// sim(a, b, t) = !(a < b t || b < a t) evaluated in double-float
__device__ __forceinline__ bool df_sim(df a, df b, df t)
{
    const df d1 = df_sub(a, df_mul(b, t));
    const df d2 = df_sub(b, df_mul(a, t));
    return !(df_sign(d1) < 0 || df_sign(d2) < 0);
}

// 8-point forward DFT of windowed column values (natural order in/out),
// radix-2 with paired FP32 butterflies; the twiddles 1 and -i are applied
// exactly, exp(-i pi/4) and exp(-3i pi/4) by complex multiplication.
__device__ __forceinline__ void dft8_fwd(const float2 (&in)[8], float2 (&out)[8])
{
    float2 a[8];
#pragma unroll
    for (int z = 0; z < 8; z++) a[z] = __fmul2_rn(in[z], make_float2(c3_wz[z], c3_wz[z]));
    // stage 1: pairs (z, z+4), twiddles exp(-2 pi i z / 8)
    float2 b[8];
#pragma unroll
    for (int z = 0; z < 4; z++) b[z] = add2(a[z], a[z + 4]);
    b[4] = sub2(a[0], a[4]);
    b[5] = cmul(sub2(a[1], a[5]), c3_tw32[4]);
    b[6] = mul_negi(sub2(a[2], a[6]));
    b[7] = cmul(sub2(a[3], a[7]), c3_tw32[12]);
    // stage 2: pairs (z, z+2) within each half, twiddles 1 and -i
    float2 c[8];
#pragma unroll
    for (int hb = 0; hb < 8; hb += 4) {
        c[hb] = add2(b[hb], b[hb + 2]);
        c[hb + 1] = add2(b[hb + 1], b[hb + 3]);
        c[hb + 2] = sub2(b[hb], b[hb + 2]);
        c[hb + 3] = mul_negi(sub2(b[hb + 1], b[hb + 3]));
    }
    // stage 3: pairs (z, z+1); outputs in bit-reversed order
    float2 d[8];
#pragma unroll
    for (int z = 0; z < 8; z += 2) {
        d[z] = add2(c[z], c[z + 1]);
        d[z + 1] = sub2(c[z], c[z + 1]);
    }
    out[0] = d[0]; out[4] = d[1]; out[2] = d[2]; out[6] = d[3];
    out[1] = d[4]; out[5] = d[5]; out[3] = d[6]; out[7] = d[7];
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
constexpr int kWarps3 = 4;
constexpr float kBoundFactor = 2.0f;   // guard band, in units of the per-bin error estimate
constexpr float kEps32 = 5.9604645e-8f;
// a + b + E^2 + rE^2 below this (with a margin for the FP32 magnitudes)
// keeps the effect of a decision under 1/4 sample unit: (4/4096) * 256 = 1/4
constexpr float kTinyPair = 65000.0f;
constexpr int kWarpSmemF2 = 8 * 5 * 32 + 2 * 2 * 5 * 32 + 32;   // float2 units per warp

struct Col {
    float2 Y[8];
    float mag[8], ab[8], E;
};

// 8-point Z DFT of one (ky, kx) column from the shared window, with its
// magnitudes, L1 magnitudes and error bound.
__device__ __forceinline__ void z_column(const float2 *win, int m, int k, int lane, float ek, Col &c)
{
    float2 col[8];
    float B = 0.f;
#pragma unroll
    for (int z = 0; z < 8; z++) {
        col[z] = win[((((2 * m + z) & 7) * 5) + k) * 32 + lane];
        B = __fmaf_rn(c3_wz[z], l1(col[z]), B);
    }
    dft8_fwd(col, c.Y);
#pragma unroll
    for (int kz = 0; kz < 8; kz++) {
        c.mag[kz] = __fmaf_rn(c.Y[kz].x, c.Y[kz].x, c.Y[kz].y * c.Y[kz].y);
        c.ab[kz] = l1(c.Y[kz]);
    }
    c.E = kBoundFactor * kEps32 * (ek + B);
}

// Mask a column, inverse-DFT it to Z slices 0, 1, 4, 5 and overlap-add:
// R(field 2m) = slice 0 + carried slice 4 of tile 2m-4, R(2m+1) = slice 1 +
// carried slice 5; then carry this tile's slices 4, 5 for frame m+2.
__device__ __forceinline__ void z_inverse(const float2 (&Y)[8], unsigned keep, float2 *carry /* [2][5][32] */,
                                          float2 *RA, float2 *RB /* [5][32] each */, int k, int lane)
{
    float2 y[8];
#pragma unroll
    for (int kz = 0; kz < 8; kz++) y[kz] = ((keep >> kz) & 1u) ? Y[kz] : make_float2(0.f, 0.f);
    const float2 E0 = add2(add2(add2(y[0], y[2]), y[4]), y[6]);
    const float2 O0 = add2(add2(add2(y[1], y[3]), y[5]), y[7]);
    // slice 1: even part y0 + i y2 - y4 - i y6; odd part with powers of exp(+i pi/4)
    const float2 E1 = make_float2(y[0].x - y[2].y - y[4].x + y[6].y, y[0].y + y[2].x - y[4].y - y[6].x);
    const float2 o1 = cmul(y[1], make_float2(c3_tw32[4].x, -c3_tw32[4].y));
    const float2 o3 = cmul(y[3], make_float2(c3_tw32[12].x, -c3_tw32[12].y));
    const float2 o5 = cmul(y[5], make_float2(c3_tw32[20].x, -c3_tw32[20].y));
    const float2 o7 = cmul(y[7], make_float2(c3_tw32[28].x, -c3_tw32[28].y));
    const float2 O1 = add2(add2(add2(o1, o3), o5), o7);
    const int i4 = k * 32 + lane, i5 = (5 + k) * 32 + lane;
    const float2 c4 = carry[i4], c5 = carry[i5];
    RA[k * 32 + lane] = add2(add2(E0, O0), c4);
    RB[k * 32 + lane] = add2(add2(E1, O1), c5);
    carry[i4] = sub2(E0, O0);
    carry[i5] = sub2(E1, O1);
}

__device__ __forceinline__ bool fsim(float a, float b, float t) { return (__fmaf_rn(-b, t, a) >= 0.f) && (__fmaf_rn(-a, t, b) >= 0.f); }

__device__ __forceinline__ bool funcertain(float a, float b, float t, float pa, float pb)
{
    return (fabsf(__fmaf_rn(-b, t, a)) <= pa + t * pb) || (fabsf(__fmaf_rn(-a, t, b)) <= pb + t * pa);
}

// Exact resolution of the guard-band decisions of one kx group inside the
// exact walk, one pair at a time, all lanes cooperating.
__device__ __forceinline__ unsigned resolve_uncertain(const T3Params &P, int m, int tileX, int tileY, int g,
                                                      int kxa, int lane, unsigned keep, unsigned unc)
{
    unsigned any = __ballot_sync(0xffffffffu, unc != 0);
    while (any) {
        const int src = __ffs(any) - 1;
        const unsigned su = __shfl_sync(0xffffffffu, unc, src);
        const int kz = __ffs(su) - 1;
        const int kyb = kappa(src);
        df mb, mr;
        exact_pair(P, m, tileX, tileY, kz, kyb, kxa, mb, mr);
        const int kzr = (10 - kz) & 7, kybr = (40 - kyb) & 31;
        bool sim = df_sim(mb, mr, thr_of(P, m, kz, kyb, kxa).d);
        if (kxa == 4) sim |= df_sim(mb, mr, thr_of(P, m, kzr, kybr, 4).d);
        if (lane == src) {
            keep = sim ? (keep | (1u << kz)) : (keep & ~(1u << kz));
            unc &= ~(1u << kz);
        }
        if (g == 2 && lane == kappa(kybr)) {   // kx = 4: the pair's other bin is a visitor too
            keep = sim ? (keep | (1u << kzr)) : (keep & ~(1u << kzr));
            unc &= ~(1u << kzr);
        }
        any = __ballot_sync(0xffffffffu, unc != 0);
    }
    return keep;
}

// Output stage of step m: inverse Y then X of output fields 2m (RA) and
// 2m + 1 (RB), and the store of each lane's row into its overlap class.
__device__ __forceinline__ void walk_store(const T3Params &P, const LaneConst &LC, const float2 *RA, const float2 *RB,
                                           int m, int tileX, int tileY, int cls)
{
    // Inverse Y then X, one kx at a time: lane (j, i) folds ky = kk and
    // kk+16 of output field 2m+j for its row parity, runs a 16-point
    // inverse DFT over the half-warp, and accumulates row i's cosine and
    // sine sums of the inverse X transform.
    float2 CS[8];   // (cosine sum, sine sum) of row i
#pragma unroll
    for (int x = 0; x < 8; x++) CS[x] = make_float2(0.f, 0.f);
    const float2 *Rj = LC.j ? RB : RA;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float2 lo_v = Rj[k * 32 + LC.i];        // R[kk]   (lane kappa^-1(kk) = i)
        const float2 hi_v = Rj[k * 32 + LC.i + 16];   // R[kk+16]
        float2 G = LC.y0 ? sub2(lo_v, hi_v) : add2(lo_v, hi_v);
        G = cmul(G, make_float2(LC.ptw.x, -LC.ptw.y));   // exp(+i pi kk y0 / 16)
        // 16-point inverse DFT, bit-reversed input -> natural order (DIT)
        int st = 3;
#pragma unroll
        for (int h = 1; h <= 8; h <<= 1, st--) {
            const bool upper = (LC.i & h) != 0;
            const float2 w = make_float2(LC.ftw[st].x, -LC.ftw[st].y);   // exp(+2 pi i r/(2h))
            const float2 o = shfl_xor2(G, h);
            const float2 t = cmul(upper ? G : o, w);
            G = upper ? sub2(o, t) : add2(G, t);
        }
#pragma unroll
        for (int x = 0; x < 8; x++) CS[x] = __ffma2_rn(G, c3_xi[k][x], CS[x]);
    }
    // Store row i of field 2m + j.
    const int L = tileY + LC.y0 + 2 * LC.i;
    if (L >= P.fafl && L <= P.lafl) {
        const int ofield = 2 * (m - P.frame_begin) + LC.j;
        float *dst = P.partial + (long long)cls * P.part_class_stride + (long long)ofield * P.part_field_stride +
                     (long long)((L >> 1) - P.fl_lo) * P.part_row_stride - P.avs;
        // tileX - avs is a multiple of 8, so an interior tile's row starts
        // on a 32-byte boundary whenever the planes' strides are multiples
        // of 4 floats and their base is 16-byte aligned: four vector stores
        const bool vec = ((P.part_row_stride | P.part_field_stride | P.part_class_stride) & 3) == 0 &&
                         (reinterpret_cast<uintptr_t>(P.partial) & 15) == 0 && tileX >= P.avs &&
                         tileX + 16 <= P.ave;
        if (vec) {
            float o[16];
#pragma unroll
            for (int x = 0; x < 8; x++) {
                o[x] = CS[x].x - CS[x].y;
                o[15 - x] = CS[x].x + CS[x].y;
            }
            float4 *d4 = reinterpret_cast<float4 *>(dst + tileX);
#pragma unroll
            for (int q = 0; q < 4; q++) d4[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        } else {
#pragma unroll
            for (int x = 0; x < 8; x++) {
                const int X0 = tileX + x, X1 = tileX + 15 - x;
                if (X0 >= P.avs && X0 < P.ave) dst[X0] = CS[x].x - CS[x].y;
                if (X1 >= P.avs && X1 < P.ave) dst[X1] = CS[x].x + CS[x].y;
            }
        }
    }
}

// TMODE: 0 = one uniform threshold, 1 = per-bin table, 2 = per-frame
// thresholds (batches of captures). EXACT = false: the walk over every work
// item, guard-band decisions taken in FP32 and recorded for
// tp3_resolve_kernel (an exact path inside this loop, however rarely taken,
// slows the whole walk by a third). EXACT = true: the walk again over the
// items tp3_resolve_kernel listed, deciding those bins exactly; it writes
// the same output locations, so its result replaces the FP32 one.
template <int TMODE, bool EXACT>
__global__ void __launch_bounds__(32 * kWarps3, 3) tpal3d_kernel(T3Params P)
{
    constexpr bool PER_BIN = (TMODE == 1);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int ntiles = P.ntx * P.nty;
    // Work items (tile position, chunk of frames); a grid smaller than the
    // item count walks them persistently.
    const unsigned nitems = EXACT ? min(P.counters[1], P.unc_cap) : (unsigned)(ntiles * P.nchunks);
    for (unsigned w = blockIdx.x * kWarps3 + warp; w < nitems; w += gridDim.x * kWarps3) {
    const int item = EXACT ? (int)P.rerun[2 * w] : (int)w;
    const int tile = item % ntiles;
    const int chunk = item / ntiles;
    const int tx = tile % P.ntx, ty = tile / P.ntx;
    const int tileX = P.tileX0 + 8 * tx;
    const int tileY = P.tileY0 + 16 * ty;
    int m0 = P.frame_begin + chunk * P.chunk_frames;
    int m1 = min(m0 + P.chunk_frames, P.frame_end);
    if (EXACT) {
        // only the steps a wrong decision at step mf reached: its own output
        // (fields 2mf, 2mf+1) and the one its carries feed (step mf + 2)
        const int mf = (int)P.rerun[2 * w + 1];
        m0 = max(m0, mf);
        m1 = min(m1, mf + 3);
    }
    const int cls = ((ty & 1) << 1) | (tx & 1);

    // Per-warp shared state (dynamic): window of field spectra, Z carries,
    // Z-stage output spectra and per-field bound terms.
    extern __shared__ float4 s_dyn[];
    float2 *wbase = reinterpret_cast<float2 *>(s_dyn) + (size_t)warp * kWarpSmemF2;
    float2 *win = wbase;                          // [8 slots][5 kx][32 lanes]
    float2 *carry_base = wbase + 8 * 5 * 32;      // [2][2 slices][5 kx][32 lanes]
    float *bnd = reinterpret_cast<float *>(carry_base + 2 * 2 * 5 * 32);   // [8 slots][8]

    const LaneConst LC = lane_const(lane, tileY, P.swap);
    const int my_ky = kappa(lane);
    const int kyr = (40 - my_ky) & 31;
    const int mirror_lane = kappa(kyr);

    // Steps m0-5 .. m0-3 only fill the window (fields 2(m0-2) .. 2(m0-2)+5);
    // steps m0-2 and m0-1 also run the Z stage for the carries; the rest output.
    for (int m = m0 - 5; m < m1; m++) {
        __syncwarp();
        forward_pair(P, m + 3, tileX, tileY, LC, lane, win, bnd);   // fields 2m+6, 2m+7
        __syncwarp();
        if (m < m0 - 2) continue;

        // Per-kx error-bound base (warp-uniform): sum_z w_z (A_z[kx] + R_z / 2)
        float ek[5];
#pragma unroll
        for (int k = 0; k < 5; k++) ek[k] = 0.f;
#pragma unroll
        for (int z = 0; z < 8; z++) {
            const float *b = bnd + 8 * ((2 * m + z) & 7);
            const float half_r = 0.5f * b[5];
#pragma unroll
            for (int k = 0; k < 5; k++) ek[k] = __fmaf_rn(c3_wz[z], b[k] + half_r, ek[k]);
        }
        float2 *carry = carry_base + (m & 1) * (2 * 5 * 32);
        const float tf_m = (TMODE == 2) ? P.frame_t2[3 * max(m, 0)] : P.t2f;   // uniform threshold of frame m

        // Z stage per kx pair: column A = kx 2+g (visited by the filter),
        // column B = its mirror kx 6-g (g = 2: kx 4 mirrors onto itself).
        // Z-stage outputs for fields 2m, 2m+1 go into those fields' window
        // slots: each column is written after it has been read.
        float2 *RA = win + ((2 * m) & 7) * 5 * 32;
        float2 *RB = win + ((2 * m + 1) & 7) * 5 * 32;
#pragma unroll 1
        for (int g = 0; g < 3; g++) {
            const int ka = g, kb = 4 - g;
            const int kxa = 2 + g;
            float rmag[8], rab[8], rE;
            Col B;
            if (g < 2) {
                z_column(win, m, kb, lane, g == 0 ? ek[4] : ek[3], B);
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    rmag[kz] = __shfl_sync(0xffffffffu, B.mag[kz], mirror_lane);
                    rab[kz] = __shfl_sync(0xffffffffu, B.ab[kz], mirror_lane);
                }
                rE = __shfl_sync(0xffffffffu, B.E, mirror_lane);
            }
            Col A;
            z_column(win, m, ka, lane, g == 0 ? ek[0] : (g == 1 ? ek[1] : ek[2]), A);
            if (g == 2) {
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    rmag[kz] = __shfl_sync(0xffffffffu, A.mag[kz], mirror_lane);
                    rab[kz] = __shfl_sync(0xffffffffu, A.ab[kz], mirror_lane);
                }
                rE = __shfl_sync(0xffffffffu, A.E, mirror_lane);
            }
            // The mirror of my column-A bin kz is bin kzr of the mirror lane's
            // column B (its column A when g = 2).
            unsigned keep = 0, unc = 0;
            // A pair too small to matter is left to FP32: toggling bins of
            // magnitudes |Y_b|, |Y_r| moves any output sample by at most
            // (2/4096)(|Y_b| + |Y_r|) <= (4/4096) sqrt(a + b + E^2 + rE^2)
            // (true magnitudes within E of the computed ones), so under
            // kTinyPair the change is below 1/4 of a composite sample unit
            // (0.38 LSB of yuv444p16, 7e-6 of yuv444ps).
            const float tiny_lim = kTinyPair - __fmaf_rn(A.E, A.E, rE * rE);
#pragma unroll
            for (int kz = 0; kz < 8; kz++) {
                const int kzr = (10 - kz) & 7;
                const float a = A.mag[kz], b = rmag[kzr];
                const float pa = 2.f * A.E * A.ab[kz] + A.E * A.E;
                const float pb = 2.f * rE * rab[kzr] + rE * rE;
                float t = tf_m;
                if (PER_BIN) t = thr_of(P, m, kz, my_ky, kxa).f;
                bool sim = fsim(a, b, t);
                bool u = funcertain(a, b, t, pa, pb);
                if (PER_BIN && g == 2) {   // kx = 4: the mirror bin visits too, with its own threshold
                    const float t2 = thr_of(P, m, kzr, kyr, 4).f;
                    sim |= fsim(a, b, t2);
                    u |= funcertain(a, b, t2, pa, pb);
                }
                // a carrier (its own mirror) is always kept
                const bool self = (g == 2) && (kz == kzr) && (my_ky == kyr);
                if (sim || self) keep |= 1u << kz;
                if (u && !self && !(a + b < tiny_lim)) unc |= 1u << kz;
            }
            // Record decisions inside the guard band for the exact passes
            // (a flat or black tile, whose bound is zero, never has any).
            if (__any_sync(0xffffffffu, unc != 0)) {
                if (EXACT) {
                    keep = resolve_uncertain(P, m, tileX, tileY, g, kxa, lane, keep, unc);
                } else {
                    unsigned slot = 0;
                    if (lane == 0) slot = atomicAdd(P.counters, 1u);
                    slot = __shfl_sync(0xffffffffu, slot, 0);
                    if (slot < P.unc_cap) {   // sized for every kx group of the launch
                        UncRecord &rec = P.unc_rec[slot];
                        if (lane == 0) {
                            rec.item = item;
                            rec.tile = tile;
                            rec.m = m;
                            rec.g = g;
                        }
                        rec.unc[lane] = (uint8_t)unc;
                        rec.keep[lane] = (uint8_t)keep;
                    }
                }
            }
            z_inverse(A.Y, keep, carry, RA, RB, ka, lane);
            if (g < 2) {
                // Column B bins are kept exactly when their mirror visit kept them.
                const unsigned mk = __shfl_sync(0xffffffffu, keep, mirror_lane);
                unsigned keepB = 0;
#pragma unroll
                for (int kz = 0; kz < 8; kz++) keepB |= ((mk >> ((10 - kz) & 7)) & 1u) << kz;
                z_inverse(B.Y, keepB, carry, RA, RB, kb, lane);
            }
        }
        __syncwarp();
        if (m < m0) continue;   // warm-up step: only the carries are needed

        walk_store(P, LC, RA, RB, m, tileX, tileY, cls);
    }
    __syncwarp();   // the next item reuses this warp's shared window
    }
}

// ---------------------------------------------------------------------------
// Learned-mask form: feature pass and apply pass
// ---------------------------------------------------------------------------
// FP32 threshold decisions of kx group g (the walk's rule without the exact
// resolution): bits kz of column A kept; the caller derives column B's.
__device__ __forceinline__ unsigned fp32_keep(const Col &A, const float (&rmag)[8], int g, int my_ky, int kyr, float t)
{
    unsigned keep = 0;
#pragma unroll
    for (int kz = 0; kz < 8; kz++) {
        const int kzr = (10 - kz) & 7;
        const bool self = (g == 2) && (kz == kzr) && (my_ky == kyr);
        if (fsim(A.mag[kz], rmag[kzr], t) || self) keep |= 1u << kz;
    }
    return keep;
}

__device__ __forceinline__ unsigned mirror_keep(unsigned keep, int mirror_lane)
{
    const unsigned mk = __shfl_sync(0xffffffffu, keep, mirror_lane);
    unsigned keepB = 0;
#pragma unroll
    for (int kz = 0; kz < 8; kz++) keepB |= ((mk >> ((10 - kz) & 7)) & 1u) << kz;
    return keepB;
}

__device__ __forceinline__ uint16_t bf16_bits(float x)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    return *reinterpret_cast<const uint16_t *>(&h);
}

// PASS 0: features (+ spectrum, + threshold decisions) of every Z tile the
// walk computes; PASS 1: the same walk with each bin scaled by its fraction
// (or, on fallback tiles, masked by the FP32 threshold decisions), then the
// inverse and overlap-add of the plain walk.
template <int PASS>
__global__ void __launch_bounds__(32 * kWarps3, 3) tpal3d_learned_kernel(T3Params P, T3Learn L)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int ntiles = P.ntx * P.nty;
    const unsigned nitems = (unsigned)(ntiles * P.nchunks);
    for (unsigned w = blockIdx.x * kWarps3 + warp; w < nitems; w += gridDim.x * kWarps3) {
    const int item = (int)w;
    const int tile = item % ntiles;
    const int chunk = item / ntiles;
    const int tx = tile % P.ntx, ty = tile / P.ntx;
    const int tileX = P.tileX0 + 8 * tx;
    const int tileY = P.tileY0 + 16 * ty;
    const int m0 = P.frame_begin + chunk * P.chunk_frames;
    const int m1 = min(m0 + P.chunk_frames, P.frame_end);
    const int cls = ((ty & 1) << 1) | (tx & 1);

    extern __shared__ float4 s_dyn[];
    float2 *wbase = reinterpret_cast<float2 *>(s_dyn) + (size_t)warp * kWarpSmemF2;
    float2 *win = wbase;
    float2 *carry_base = wbase + 8 * 5 * 32;
    float *bnd = reinterpret_cast<float *>(carry_base + 2 * 2 * 5 * 32);

    const LaneConst LC = lane_const(lane, tileY, P.swap);
    const int my_ky = kappa(lane);
    const int kyr = (40 - my_ky) & 31;
    const int mirror_lane = kappa(kyr);

    for (int m = m0 - 5; m < m1; m++) {
        __syncwarp();
        forward_pair(P, m + 3, tileX, tileY, LC, lane, win, bnd);
        __syncwarp();
        if (m < m0 - 2) continue;
        const long long base = ((long long)(m - L.z0) * ntiles + tile) * 1280;
        float2 *carry = carry_base + (m & 1) * (2 * 5 * 32);
        float2 *RA = win + ((2 * m) & 7) * 5 * 32;
        float2 *RB = win + ((2 * m + 1) & 7) * 5 * 32;
        const bool fb = (PASS == 1) ? (L.fallback[(long long)(m - L.z0) * ntiles + tile] != 0) : false;
#pragma unroll 1
        for (int g = 0; g < 3; g++) {
            const int ka = g, kb = 4 - g;
            float rmag[8];
            Col B;
            if (g < 2) {
                z_column(win, m, kb, lane, 0.f, B);
#pragma unroll
                for (int kz = 0; kz < 8; kz++) rmag[kz] = __shfl_sync(0xffffffffu, B.mag[kz], mirror_lane);
            }
            Col A;
            z_column(win, m, ka, lane, 0.f, A);
            if (g == 2) {
#pragma unroll
                for (int kz = 0; kz < 8; kz++) rmag[kz] = __shfl_sync(0xffffffffu, A.mag[kz], mirror_lane);
            }
            if (PASS == 0) {
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    const long long va = base + (ka * 8 + kz) * 32 + my_ky;
                    L.feat[va] = bf16_bits(log1pf(sqrtf(A.mag[kz])) * 0.0625f);
                    if (L.spec != nullptr) L.spec[va] = A.Y[kz];
                    if (g < 2) {
                        const long long vb = base + (kb * 8 + kz) * 32 + my_ky;
                        L.feat[vb] = bf16_bits(log1pf(sqrtf(B.mag[kz])) * 0.0625f);
                        if (L.spec != nullptr) L.spec[vb] = B.Y[kz];
                    }
                }
                if (L.plain_p != nullptr) {
                    const unsigned keep = fp32_keep(A, rmag, g, my_ky, kyr, P.t2f);
                    const unsigned keepB = mirror_keep(keep, mirror_lane);
#pragma unroll
                    for (int kz = 0; kz < 8; kz++) {
                        L.plain_p[base + (ka * 8 + kz) * 32 + my_ky] = (float)((keep >> kz) & 1u);
                        if (g < 2) L.plain_p[base + (kb * 8 + kz) * 32 + my_ky] = (float)((keepB >> kz) & 1u);
                    }
                }
            } else {
                if (fb) {
                    const unsigned keep = fp32_keep(A, rmag, g, my_ky, kyr, P.t2f);
                    const unsigned keepB = mirror_keep(keep, mirror_lane);
                    z_inverse(A.Y, keep, carry, RA, RB, ka, lane);
                    if (g < 2) z_inverse(B.Y, keepB, carry, RA, RB, kb, lane);
                } else {
#pragma unroll
                    for (int kz = 0; kz < 8; kz++) {
                        const float pa = __ldg(L.p + base + (ka * 8 + kz) * 32 + my_ky);
                        A.Y[kz] = __fmul2_rn(A.Y[kz], make_float2(pa, pa));
                        if (g < 2) {
                            const float pb = __ldg(L.p + base + (kb * 8 + kz) * 32 + my_ky);
                            B.Y[kz] = __fmul2_rn(B.Y[kz], make_float2(pb, pb));
                        }
                    }
                    z_inverse(A.Y, 0xFFu, carry, RA, RB, ka, lane);
                    if (g < 2) z_inverse(B.Y, 0xFFu, carry, RA, RB, kb, lane);
                }
            }
        }
        __syncwarp();
        if (PASS == 0 || m < m0) continue;
        walk_store(P, LC, RA, RB, m, tileX, tileY, cls);
    }
    __syncwarp();
    }
}

int tp3_learned_launch(const T3Params &P, const T3Learn &L, int pass, cudaStream_t stream)
{
    const long long items = (long long)P.ntx * P.nty * P.nchunks;
    if (items <= 0) return 0;
    const unsigned blocks = (unsigned)((items + kWarps3 - 1) / kWarps3);
    const size_t smem = sizeof(float2) * (size_t)kWarpSmemF2 * kWarps3;
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return -1;
    if (!attr_set[dev]) {
        const auto a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (cudaFuncSetAttribute(tpal3d_learned_kernel<0>, a, (int)smem) != cudaSuccess ||
            cudaFuncSetAttribute(tpal3d_learned_kernel<1>, a, (int)smem) != cudaSuccess)
            return -1;
        attr_set[dev] = true;
    }
    if (pass == 0) {
        if (L.feat == nullptr) return -1;
        tpal3d_learned_kernel<0><<<blocks, 32 * kWarps3, smem, stream>>>(P, L);
    } else {
        if (L.p == nullptr || L.fallback == nullptr || P.partial == nullptr) return -1;
        tpal3d_learned_kernel<1><<<blocks, 32 * kWarps3, smem, stream>>>(P, L);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------------------
// Deferred exact decisions
// ---------------------------------------------------------------------------
// One warp per record: decide its guard-band bins exactly in double-float
// (the arithmetic of exact_pair, with the X stage of the record's two kx
// columns computed once for all its bins) and, where an exact decision
// differs from the FP32 one the walk used, list the record's work item and
// step for the exact walk.
__global__ void __launch_bounds__(32 * kWarps3) tp3_resolve_kernel(T3Params P)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned n = min(P.counters[0], P.unc_cap);
    unsigned n_exact = 0, n_flip = 0;
    const int z = lane >> 2, part = lane & 3;
    // Window-scaled double-float twiddles, w_y(y) exp(-2 pi i r/32) for every
    // (y, r) and w_z(z) exp(-2 pi i 4 r/32) for every (z, r), formed once per
    // block with the same df_mul the products would use (the same values),
    // read from shared memory: a warp reads them with 8 distinct indices,
    // which the constant cache would serialise. Rows padded by one entry.
    __shared__ float4 s_yw[32][33], s_zw[8][8];
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int y = i >> 5, r = i & 31;
        const df w = {c3_dfwy[y][0], c3_dfwy[y][1]};
        const df re = df_mul({c3_dftw32[r][0], c3_dftw32[r][1]}, w), im = df_mul({c3_dftw32[r][2], c3_dftw32[r][3]}, w);
        s_yw[y][r] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
    for (int i = threadIdx.x; i < 8 * 8; i += blockDim.x) {
        const int zz = i >> 3, r = i & 7;
        const df w = {c3_dfwz[zz][0], c3_dfwz[zz][1]};
        const df re = df_mul({c3_dftw32[4 * r][0], c3_dftw32[4 * r][1]}, w);
        const df im = df_mul({c3_dftw32[4 * r][2], c3_dftw32[4 * r][3]}, w);
        s_zw[zz][r] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
    __syncthreads();
    auto as_dfc = [](float4 v) -> dfc { return {{v.x, v.y}, {v.z, v.w}}; };
    for (unsigned rec = blockIdx.x * kWarps3 + warp; rec < n; rec += gridDim.x * kWarps3) {
        const UncRecord &R = P.unc_rec[rec];
        const int item = R.item, tile = R.tile, m = R.m, g = R.g;
        const int tileX = P.tileX0 + 8 * (tile % P.ntx), tileY = P.tileY0 + 16 * (tile / P.ntx);
        const int kxa = 2 + g;
        const unsigned keep = R.keep[lane];
        unsigned unc = R.unc[lane];
        // X stage of this lane's four rows of field 2m + z, both columns
        const int f = 2 * m + z;
        const int p = (f & 1) ^ P.swap;
        const int y0 = (p - tileY) & 1;
        dfc xa[4], xb[4];
        const uint16_t *fp = (f >= 0 && f < P.nfields) ? field_at(P, f) : nullptr;
#pragma unroll
        for (int r4 = 0; r4 < 4; r4++) {
            xa[r4] = xb[r4] = {{0.f, 0.f}, {0.f, 0.f}};
            const int L = tileY + y0 + 2 * (part * 4 + r4);
            if (fp == nullptr || L < P.fafl || L > P.lafl) continue;
            const long long base = (long long)(L >> 1) * P.fw + tileX;   // within the field
            x_row_pair(fp, base, (long long)P.fh * P.fw, P.black, kxa, xa[r4], xb[r4]);
        }
        bool flipped = false;
        unsigned any = __ballot_sync(0xffffffffu, unc != 0);
        while (any) {
            const int src = __ffs(any) - 1;
            const unsigned su = __shfl_sync(0xffffffffu, unc, src);
            const int kz = __ffs(su) - 1;
            const int kyb = kappa(src);
            const int kzr = (10 - kz) & 7, kybr = (40 - kyb) & 31;
            // Y stage over this lane's rows, then the 4 row groups, then Z
            dfc accb = {{0.f, 0.f}, {0.f, 0.f}}, accr = accb;
#pragma unroll
            for (int r4 = 0; r4 < 4; r4++) {
                const int y = y0 + 2 * (part * 4 + r4);
                const dfc cb = as_dfc(s_yw[y][(kyb * y) & 31]), cr = as_dfc(s_yw[y][(kybr * y) & 31]);
                accb = dfc_add(accb, dfc_mul(xa[r4], cb));
                accr = dfc_add(accr, dfc_mul(xb[r4], cr));
            }
            accb = dfc_add(accb, dfc_shfl_xor(accb, 1));
            accb = dfc_add(accb, dfc_shfl_xor(accb, 2));
            accr = dfc_add(accr, dfc_shfl_xor(accr, 1));
            accr = dfc_add(accr, dfc_shfl_xor(accr, 2));
            {
                const dfc tb = as_dfc(s_zw[z][(kz * z) & 7]), tr = as_dfc(s_zw[z][(kzr * z) & 7]);
                accb = dfc_mul(accb, tb);
                accr = dfc_mul(accr, tr);
            }
            accb = dfc_add(accb, dfc_shfl_xor(accb, 4));
            accb = dfc_add(accb, dfc_shfl_xor(accb, 8));
            accb = dfc_add(accb, dfc_shfl_xor(accb, 16));
            accr = dfc_add(accr, dfc_shfl_xor(accr, 4));
            accr = dfc_add(accr, dfc_shfl_xor(accr, 8));
            accr = dfc_add(accr, dfc_shfl_xor(accr, 16));
            const df mb = dfc_abs2(accb), mr = dfc_abs2(accr);
            bool sim = df_sim(mb, mr, thr_of(P, m, kz, kyb, kxa).d);
            if (kxa == 4) sim |= df_sim(mb, mr, thr_of(P, m, kzr, kybr, 4).d);
            const bool old = ((__shfl_sync(0xffffffffu, keep, src) >> kz) & 1u) != 0;
            flipped |= (old != sim);
            if (lane == src) {
                n_exact++;
                if (old != sim) n_flip++;
                unc &= ~(1u << kz);
            }
            if (g == 2 && lane == kappa(kybr)) unc &= ~(1u << kzr);   // kx = 4: the same pair
            any = __ballot_sync(0xffffffffu, unc != 0);
        }
        if (flipped && lane == 0) {
            const unsigned at = atomicAdd(P.counters + 1, 1u);
            if (at < P.unc_cap) {   // at most one entry per record
                P.rerun[2 * at] = (unsigned)item;
                P.rerun[2 * at + 1] = (unsigned)m;
            }
        }
    }
    if (P.stats != nullptr) {
        if (n_exact) atomicAdd(P.stats + 0, n_exact);
        if (n_flip) atomicAdd(P.stats + 1, n_flip);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static double rc_window(int n, int N) { return 0.5 - (0.5 * cos((2 * M_PI * (n + 0.5)) / N)); }

static void split_df(double v, float &hi, float &lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

int tp3_init_constants(int device)
{
    if (device >= 0 && device < 64 && g_tp3_constants_ready[device]) return 0;
    float cwx[5][8], swx[5][8], cix[5][8], six[5][8];
    for (int k = 0; k < 5; k++) {
        const int kx = k + 2;
        for (int x = 0; x < 8; x++) {
            const double th = 2.0 * M_PI * kx * (x - 7.5) / 16.0;
            const double w = rc_window(x, 16);
            cwx[k][x] = (float)(w * cos(th));
            swx[k][x] = (float)(w * sin(th));
            cix[k][x] = (float)((2.0 / 4096.0) * cos(th));
            six[k][x] = (float)((2.0 / 4096.0) * sin(th));
        }
    }
    float wy[2][16], wx[16], wz[8];
    for (int y0 = 0; y0 < 2; y0++)
        for (int i = 0; i < 16; i++) wy[y0][i] = (float)rc_window(y0 + 2 * i, 32);
    for (int x = 0; x < 16; x++) wx[x] = (float)rc_window(x, 16);
    for (int z = 0; z < 8; z++) wz[z] = (float)rc_window(z, 8);
    float2 tw16[16], tw32[32];
    for (int r = 0; r < 16; r++) tw16[r] = make_float2((float)cos(-2 * M_PI * r / 16), (float)sin(-2 * M_PI * r / 16));
    for (int r = 0; r < 32; r++) tw32[r] = make_float2((float)cos(-2 * M_PI * r / 32), (float)sin(-2 * M_PI * r / 32));
    float dfwy[32][2], dfwz[8][2], dftw32[32][4];
    int qx[5][16][4];
    for (int k = 0; k < 5; k++)
        for (int x = 0; x < 16; x++) {
            const double w = rc_window(x, 16);
            const double a = -2.0 * M_PI * (k + 2) * x / 16.0;
            const double parts[2] = {w * cos(a), w * sin(a)};
            for (int c = 0; c < 2; c++) {
                const long long q = llround(parts[c] * 1152921504606846976.0);   // 2^60
                qx[k][x][2 * c] = (int)(q >> 30);                               // floor(q / 2^30)
                qx[k][x][2 * c + 1] = (int)(q & ((1LL << 30) - 1));
            }
        }
    for (int y = 0; y < 32; y++) split_df(rc_window(y, 32), dfwy[y][0], dfwy[y][1]);
    for (int z = 0; z < 8; z++) split_df(rc_window(z, 8), dfwz[z][0], dfwz[z][1]);
    for (int r = 0; r < 32; r++) {
        split_df(cos(-2 * M_PI * r / 32), dftw32[r][0], dftw32[r][1]);
        split_df(sin(-2 * M_PI * r / 32), dftw32[r][2], dftw32[r][3]);
    }
#define TPAL_CPY(sym, src)                                                  \
    if (cudaMemcpyToSymbol(sym, src, sizeof(src)) != cudaSuccess) return -1;
    float2 xf[5][8], xi[5][8];
    for (int k = 0; k < 5; k++)
        for (int x = 0; x < 8; x++) {
            xf[k][x] = make_float2(cwx[k][x], -swx[k][x]);
            xi[k][x] = make_float2(cix[k][x], six[k][x]);
        }
    TPAL_CPY(c3_xf, xf);
    TPAL_CPY(c3_xi, xi);
    TPAL_CPY(c3_wy, wy);
    TPAL_CPY(c3_wx, wx);
    TPAL_CPY(c3_wz, wz);
    TPAL_CPY(c3_tw16, tw16);
    TPAL_CPY(c3_tw32, tw32);
    TPAL_CPY(c3_qx, qx);
    TPAL_CPY(c3_dfwy, dfwy);
    TPAL_CPY(c3_dfwz, dfwz);
    TPAL_CPY(c3_dftw32, dftw32);
#undef TPAL_CPY
    if (device >= 0 && device < 64) g_tp3_constants_ready[device] = true;
    return 0;
}

int tp3_launch(const T3Params &P, cudaStream_t stream, int max_blocks)
{
    const long long items = (long long)P.ntx * P.nty * P.nchunks;
    if (items <= 0) return 0;
    unsigned blocks = (unsigned)((items + kWarps3 - 1) / kWarps3);
    if (max_blocks > 0 && blocks > (unsigned)max_blocks) blocks = (unsigned)max_blocks;   // persistent grid
    const size_t smem = sizeof(float2) * (size_t)kWarpSmemF2 * kWarps3;
    // function attributes are per device
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return -1;
    if (!attr_set[dev]) {
        const int b = (int)smem;
        const auto a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (cudaFuncSetAttribute(tpal3d_kernel<0, false>, a, b) != cudaSuccess ||
            cudaFuncSetAttribute(tpal3d_kernel<1, false>, a, b) != cudaSuccess ||
            cudaFuncSetAttribute(tpal3d_kernel<2, false>, a, b) != cudaSuccess ||
            cudaFuncSetAttribute(tpal3d_kernel<0, true>, a, b) != cudaSuccess ||
            cudaFuncSetAttribute(tpal3d_kernel<1, true>, a, b) != cudaSuccess ||
            cudaFuncSetAttribute(tpal3d_kernel<2, true>, a, b) != cudaSuccess)
            return -1;
        attr_set[dev] = true;
    }
    if (P.unc_rec == nullptr || P.counters == nullptr || P.rerun == nullptr) return -1;
    const unsigned t = 32 * kWarps3;
    if (P.thr_table != nullptr) tpal3d_kernel<1, false><<<blocks, t, smem, stream>>>(P);
    else if (P.frame_t2 != nullptr) tpal3d_kernel<2, false><<<blocks, t, smem, stream>>>(P);
    else tpal3d_kernel<0, false><<<blocks, t, smem, stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int tp3_resolve_launch(const T3Params &P, cudaStream_t stream)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    // the record and item counts are only known on the device: fixed grids
    // walk them
    tp3_resolve_kernel<<<4 * sms, 32 * kWarps3, 0, stream>>>(P);
    const size_t smem = sizeof(float2) * (size_t)kWarpSmemF2 * kWarps3;
    const unsigned t = 32 * kWarps3, blocks = 3u * (unsigned)sms;
    if (P.thr_table != nullptr) tpal3d_kernel<1, true><<<blocks, t, smem, stream>>>(P);
    else if (P.frame_t2 != nullptr) tpal3d_kernel<2, true><<<blocks, t, smem, stream>>>(P);
    else tpal3d_kernel<0, true><<<blocks, t, smem, stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace tpal
