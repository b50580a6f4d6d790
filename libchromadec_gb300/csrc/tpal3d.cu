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
#include <cuda_runtime.h>

#include "tpal_common.cuh"
#include "tpal_kernels.h"

namespace tpal {

// ---------------------------------------------------------------------------
// Constant tables (filled by tp3_init_constants from double precision)
// ---------------------------------------------------------------------------
__constant__ float c3_cwx[5][8];   // forward X: w(x) cos(theta_kx), theta = 2 pi kx (x - 7.5) / 16
__constant__ float c3_swx[5][8];   // forward X: w(x) sin(theta_kx)
__constant__ float c3_cix[5][8];   // inverse X: (2/4096) cos(theta)
__constant__ float c3_six[5][8];   // inverse X: (2/4096) sin(theta)
__constant__ float c3_wy[2][16];   // w_y(y0 + 2i), 32-point raised cosine
__constant__ float c3_wx[16];      // w_x(x)
__constant__ float c3_wz[8];       // w_z(z)
__constant__ float2 c3_tw16[16];   // exp(-2 pi i r / 16)
__constant__ float2 c3_tw32[32];   // exp(-2 pi i r / 32)
// double-float tables for the exact decision path
__constant__ float c3_dfx[5][16][4];   // w_x(x) exp(-2 pi i kx x/16): re.hi, re.lo, im.hi, im.lo
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

__device__ __forceinline__ Thr thr_of(const T3Params &P, int kz, int ky, int kx)
{
    if (P.thr_table == nullptr) return {P.t2f, {P.t2hi, P.t2lo}};
    const float *t = P.thr_table + 3 * ((kz * 32 + ky) * 3 + (kx - 2));
    return {t[0], {t[1], t[2]}};
}

// ---------------------------------------------------------------------------
// Forward X and Y stages for two consecutive fields (2q, 2q+1).
// On return lane l holds S_{2q}[kappa(l)][kx] in s0 and S_{2q+1}[kappa(l)][kx]
// in s1 (kx = 2..6), and the smem bound slots of both fields are written.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void forward_pair(const T3Params &P, int q, int tileX, int tileY, int lane,
                                             float2 (&s0)[5], float2 (&s1)[5], float *bnd /* [8][8] */)
{
    const int j = lane >> 4;
    const int i = lane & 15;
    const int f = 2 * q + j;
    const int p = f & 1;                  // field offset: even index = first field
    const int y0 = (p - tileY) & 1;       // frame-row parity of this field's rows in the tile
    const int y = y0 + 2 * i;
    const int L = tileY + y;              // frame line
    const bool valid = (f >= 0) && (f < P.nfields) && (L >= P.fafl) && (L <= P.lafl);

    float2 X[5];
#pragma unroll
    for (int k = 0; k < 5; k++) X[k] = make_float2(0.0f, 0.0f);
    float rowl1 = 0.0f;
    if (valid) {
        const long long base = (long long)(f - P.field_base) * P.field_stride + (long long)(L >> 1) * P.fw + tileX;
        int a[16];
        int sum = 0;
#pragma unroll
        for (int x = 0; x < 16; x++) {
            long long idx = base + x;
            idx = idx < 0 ? 0 : idx;
            a[x] = (int)__ldg(P.fields + idx) - P.black;
            sum += a[x];
        }
        // s_x = a_x + a_15-x - 2*mean, d_x = a_x - a_15-x (both exact in FP32)
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const float sx = (float)(8 * (a[x] + a[15 - x]) - sum) * 0.125f;
            const float dx = (float)(a[x] - a[15 - x]);
#pragma unroll
            for (int k = 0; k < 5; k++) {
                X[k].x = __fmaf_rn(c3_cwx[k][x], sx, X[k].x);
                X[k].y = __fmaf_rn(-c3_swx[k][x], dx, X[k].y);
            }
            const float m16 = (float)sum * 0.0625f;
            rowl1 = __fmaf_rn(c3_wx[x], fabsf((float)a[x] - m16) + fabsf((float)a[15 - x] - m16), rowl1);
        }
    }
    const float wy = c3_wy[y0][i];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        X[k].x *= wy;
        X[k].y *= wy;
    }
    rowl1 *= wy;

    // Bound terms: per field and kx, sum over rows of |X|_1; and the row-L1 sum.
    float A[6];
#pragma unroll
    for (int k = 0; k < 5; k++) A[k] = l1(X[k]);
    A[5] = rowl1;
#pragma unroll
    for (int h = 1; h < 16; h <<= 1) {
#pragma unroll
        for (int k = 0; k < 6; k++) A[k] += __shfl_xor_sync(0xffffffffu, A[k], h);
    }
    if (i == 0) {
        float *b = bnd + 8 * (f & 7);
#pragma unroll
        for (int k = 0; k < 6; k++) b[k] = A[k];
    }

    // 16-point forward DFT over the rows of each half-warp (radix-2 DIF,
    // bit-reversed output: lane i ends up with bin rev4(i)).
#pragma unroll
    for (int h = 8; h >= 1; h >>= 1) {
        const bool upper = (i & h) != 0;
        const int r = i & (h - 1);
        const float2 w = c3_tw16[r * (8 / h)];   // exp(-2 pi i r / (2h))
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const float2 o = shfl_xor2(X[k], h);
            if (upper) {
                X[k] = cmul(make_float2(o.x - X[k].x, o.y - X[k].y), w);
            } else {
                X[k] = make_float2(X[k].x + o.x, X[k].y + o.y);
            }
        }
    }
    // Parity twiddle: S[kk] = exp(-2 pi i kk y0/32) A[kk], S[kk+16] = (-1)^y0 S[kk]
    const int kk = rev4(i);
    const float2 tw = y0 ? c3_tw32[kk] : make_float2(1.0f, 0.0f);
    float2 lo[5], hi[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        lo[k] = cmul(X[k], tw);
        hi[k] = y0 ? make_float2(-lo[k].x, -lo[k].y) : lo[k];
    }
    // Exchange halves so lane l holds both fields at ky = kappa(l).
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float2 send = j ? lo[k] : hi[k];
        const float2 recv = shfl_xor2(send, 16);
        s0[k] = j ? recv : lo[k];
        s1[k] = j ? hi[k] : recv;
    }
}

// ---------------------------------------------------------------------------
// Exact (double-float) magnitudes of bin b = (kzb, kyb, kxb) and its mirror
// r of Z tile T(2m). All 32 lanes cooperate; every lane returns the result.
// ---------------------------------------------------------------------------
__device__ __noinline__ void exact_pair(const T3Params &P, int m, int tileX, int tileY, int kzb, int kyb, int kxb,
                                        df &mb, df &mr)
{
    const int lane = threadIdx.x & 31;
    const int kzr = (10 - kzb) & 7, kyr = (40 - kyb) & 31, kxr = 8 - kxb;
    const int z = lane >> 2;
    const int part = lane & 3;
    const int f = 2 * m + z;
    const int p = f & 1;
    const int y0 = (p - tileY) & 1;
    dfc accb = {{0.f, 0.f}, {0.f, 0.f}}, accr = accb;
    if (f >= 0 && f < P.nfields) {
        for (int r4 = 0; r4 < 4; r4++) {
            const int i = part * 4 + r4;
            const int y = y0 + 2 * i;
            const int L = tileY + y;
            if (L < P.fafl || L > P.lafl) continue;
            const long long base = (long long)(f - P.field_base) * P.field_stride + (long long)(L >> 1) * P.fw + tileX;
            dfc xb = {{0.f, 0.f}, {0.f, 0.f}}, xr = xb;
            for (int x = 0; x < 16; x++) {
                long long idx = base + x;
                idx = idx < 0 ? 0 : idx;
                const float a = (float)((int)__ldg(P.fields + idx) - P.black);
                const float *cb = c3_dfx[kxb - 2][x];
                const float *cr = c3_dfx[kxr - 2][x];
                xb.re = df_add(xb.re, df_mul_f({cb[0], cb[1]}, a));
                xb.im = df_add(xb.im, df_mul_f({cb[2], cb[3]}, a));
                xr.re = df_add(xr.re, df_mul_f({cr[0], cr[1]}, a));
                xr.im = df_add(xr.im, df_mul_f({cr[2], cr[3]}, a));
            }
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

// 8-point forward DFT of windowed column values (natural order in/out).
__device__ __forceinline__ void dft8_fwd(const float2 (&in)[8], float2 (&out)[8])
{
    float2 a[8];
#pragma unroll
    for (int z = 0; z < 8; z++) a[z] = make_float2(in[z].x * c3_wz[z], in[z].y * c3_wz[z]);
    // stage 1: pairs (z, z+4)
    float2 b[8];
#pragma unroll
    for (int z = 0; z < 4; z++) {
        b[z] = make_float2(a[z].x + a[z + 4].x, a[z].y + a[z + 4].y);
        const float2 d = make_float2(a[z].x - a[z + 4].x, a[z].y - a[z + 4].y);
        b[z + 4] = cmul(d, c3_tw32[4 * z]);   // exp(-2 pi i z / 8)
    }
    // stage 2: pairs (z, z+2) within each half
    float2 c[8];
#pragma unroll
    for (int hb = 0; hb < 8; hb += 4) {
#pragma unroll
        for (int z = 0; z < 2; z++) {
            const float2 u = b[hb + z], v = b[hb + z + 2];
            c[hb + z] = make_float2(u.x + v.x, u.y + v.y);
            const float2 d = make_float2(u.x - v.x, u.y - v.y);
            c[hb + z + 2] = cmul(d, c3_tw32[8 * z]);   // exp(-2 pi i z / 4)
        }
    }
    // stage 3: pairs (z, z+1); outputs in bit-reversed order
    float2 d[8];
#pragma unroll
    for (int z = 0; z < 8; z += 2) {
        d[z] = make_float2(c[z].x + c[z + 1].x, c[z].y + c[z + 1].y);
        d[z + 1] = make_float2(c[z].x - c[z + 1].x, c[z].y - c[z + 1].y);
    }
    out[0] = d[0]; out[4] = d[1]; out[2] = d[2]; out[6] = d[3];
    out[1] = d[4]; out[5] = d[5]; out[3] = d[6]; out[7] = d[7];
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
constexpr int kWarps3 = 4;
constexpr float kBoundFactor = 2.0f;   // guard band, in units of the per-bin error estimate

__global__ void __launch_bounds__(32 * kWarps3) tpal3d_kernel(T3Params P)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int ntiles = P.ntx * P.nty;
    const int item = blockIdx.x * kWarps3 + warp;
    if (item >= ntiles * P.nchunks) return;
    const int tile = item % ntiles;
    const int chunk = item / ntiles;
    const int tx = tile % P.ntx, ty = tile / P.ntx;
    const int tileX = P.tileX0 + 8 * tx;
    const int tileY = P.tileY0 + 16 * ty;
    const int m0 = P.frame_begin + chunk * P.chunk_frames;
    const int m1 = min(m0 + P.chunk_frames, P.frame_end);
    const int cls = ((ty & 1) << 1) | (tx & 1);

    __shared__ float s_bnd[kWarps3][8 * 8];
    __shared__ float2 s_carry[kWarps3][2][2][5][32];
    float *bnd = s_bnd[warp];

    const int my_ky = kappa(lane);
    const int mirror_lane = kappa((40 - my_ky) & 31);

    // S window: sw[z] = S of field 2m + z at ky = kappa(lane)
    float2 sw[8][5];
#pragma unroll
    for (int z = 0; z < 8; z++)
#pragma unroll
        for (int k = 0; k < 5; k++) sw[z][k] = make_float2(0.f, 0.f);

    // Prefill fields 2(m0-2) .. 2(m0-2)+5
    for (int q = m0 - 2; q < m0 + 1; q++) {
#pragma unroll
        for (int z = 0; z < 6; z++)
#pragma unroll
            for (int k = 0; k < 5; k++) sw[z][k] = sw[z + 2][k];
        forward_pair(P, q, tileX, tileY, lane, sw[6], sw[7], bnd);
    }

    unsigned int n_exact = 0, n_flip = 0;

    for (int m = m0 - 2; m < m1; m++) {
        __syncwarp();
        // Slide the window and add fields 2m+6, 2m+7.
#pragma unroll
        for (int z = 0; z < 6; z++)
#pragma unroll
            for (int k = 0; k < 5; k++) sw[z][k] = sw[z + 2][k];
        forward_pair(P, m + 3, tileX, tileY, lane, sw[6], sw[7], bnd);
        __syncwarp();

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

        float2 RA[5], RB[5];   // spectra of output fields 2m (A) and 2m+1 (B)
        const int slot = m & 1;

        // Z stage, per kx group: (2,6), (3,5), (4)
#pragma unroll
        for (int g = 0; g < 3; g++) {
            const int ncol = (g < 2) ? 2 : 1;
            const int kxs[2] = {2 + g, 6 - g};
            float2 Y[2][8];
            float mag[2][8], ab[2][8], E[2];
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (c >= ncol) break;
                const int k = kxs[c] - 2;
                float2 col[8];
                float B = 0.f;
#pragma unroll
                for (int z = 0; z < 8; z++) {
                    col[z] = sw[z][k];
                    B = __fmaf_rn(c3_wz[z], l1(sw[z][k]), B);
                }
                dft8_fwd(col, Y[c]);
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    mag[c][kz] = __fmaf_rn(Y[c][kz].x, Y[c][kz].x, Y[c][kz].y * Y[c][kz].y);
                    ab[c][kz] = l1(Y[c][kz]);
                }
                E[c] = kBoundFactor * 5.9604645e-8f * (ek[k] + B);
            }
            // Mirror column data from the mirror lane: for my column c the
            // mirror column is 8 - kx, held by the mirror lane as its column
            // (ncol == 2 ? 1 - c : 0).
            float rmag[2][8], rab[2][8], rE[2];
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (c >= ncol) break;
                const int src_c = (ncol == 2) ? 1 - c : 0;
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    rmag[c][kz] = __shfl_sync(0xffffffffu, mag[src_c][kz], mirror_lane);
                    rab[c][kz] = __shfl_sync(0xffffffffu, ab[src_c][kz], mirror_lane);
                }
                rE[c] = __shfl_sync(0xffffffffu, E[src_c], mirror_lane);
            }
            // Decisions
            unsigned keep = 0, unc = 0;   // bit c*8 + kz
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (c >= ncol) break;
                const int kx = kxs[c];
#pragma unroll
                for (int kz = 0; kz < 8; kz++) {
                    const int kzr = (10 - kz) & 7;
                    const int bit = c * 8 + kz;
                    const int kyr = (40 - my_ky) & 31;
                    if (kx == 4 && kz == kzr && my_ky == kyr) {   // its own mirror: a carrier
                        keep |= 1u << bit;
                        continue;
                    }
                    const float a = mag[c][kz], b = rmag[c][kzr];
                    const float Ea = E[c], Eb = rE[c];
                    const float pa = 2.f * Ea * ab[c][kz] + Ea * Ea;
                    const float pb = 2.f * Eb * rab[c][kzr] + Eb * Eb;
                    bool sim = false, u = false;
#pragma unroll
                    for (int v = 0; v < 2; v++) {
                        // visit 0: this bin visits (kx <= 4); visit 1: the mirror visits (kx >= 4)
                        if (v == 0 && kx > 4) continue;
                        if (v == 1 && kx < 4) continue;
                        const Thr t = (v == 0) ? thr_of(P, kz, my_ky, kx) : thr_of(P, kzr, kyr, 8 - kx);
                        const float d1 = __fmaf_rn(-b, t.f, a);
                        const float d2 = __fmaf_rn(-a, t.f, b);
                        sim |= (d1 >= 0.f) && (d2 >= 0.f);
                        u |= (fabsf(d1) <= pa + t.f * pb) || (fabsf(d2) <= pb + t.f * pa);
                    }
                    if (sim) keep |= 1u << bit;
                    if (u) unc |= 1u << bit;
                }
            }
            // Resolve uncertain decisions exactly (rare): one pair at a time.
            unsigned any = __ballot_sync(0xffffffffu, unc != 0);
            while (any) {
                const int src = __ffs(any) - 1;
                const unsigned su = __shfl_sync(0xffffffffu, unc, src);
                const int bit = __ffs(su) - 1;
                const int c = bit >> 3, kz = bit & 7;
                const int kxb = (c == 0) ? 2 + g : 6 - g;
                const int kyb = kappa(src);
                df mb, mr;
                exact_pair(P, m, tileX, tileY, kz, kyb, kxb, mb, mr);
                const int kzr = (10 - kz) & 7, kyr = (40 - kyb) & 31, kxr = 8 - kxb;
                bool sim = false;
                if (kxb <= 4) sim |= df_sim(mb, mr, thr_of(P, kz, kyb, kxb).d);
                if (kxb >= 4) sim |= df_sim(mb, mr, thr_of(P, kzr, kyr, kxr).d);
                // update the owning lane of b and of its mirror r
                const int rl = kappa(kyr);
                const int rc = (ncol == 2) ? 1 - c : 0;
                const int rbit = rc * 8 + kzr;
                if (lane == src) {
                    const bool was = (keep >> bit) & 1u;
                    n_exact++;
                    if (was != sim) n_flip++;
                    keep = sim ? (keep | (1u << bit)) : (keep & ~(1u << bit));
                    unc &= ~(1u << bit);
                }
                if (lane == rl) {
                    keep = sim ? (keep | (1u << rbit)) : (keep & ~(1u << rbit));
                    unc &= ~(1u << rbit);
                }
                any = __ballot_sync(0xffffffffu, unc != 0);
            }
            // Mask, inverse Z to slices 0, 1, 4, 5, and Z overlap-add.
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (c >= ncol) break;
                const int k = kxs[c] - 2;
                float2 y[8];
#pragma unroll
                for (int kz = 0; kz < 8; kz++)
                    y[kz] = ((keep >> (c * 8 + kz)) & 1u) ? Y[c][kz] : make_float2(0.f, 0.f);
                const float2 E0 = make_float2(y[0].x + y[2].x + y[4].x + y[6].x, y[0].y + y[2].y + y[4].y + y[6].y);
                const float2 O0 = make_float2(y[1].x + y[3].x + y[5].x + y[7].x, y[1].y + y[3].y + y[5].y + y[7].y);
                // z = 1: even part y0 + i y2 - y4 - i y6; odd part with w = exp(+i pi/4)
                const float2 E1 = make_float2(y[0].x - y[2].y - y[4].x + y[6].y, y[0].y + y[2].x - y[4].y - y[6].x);
                const float2 o1 = cmul(y[1], make_float2(c3_tw32[4].x, -c3_tw32[4].y));    // w
                const float2 o3 = cmul(y[3], make_float2(c3_tw32[12].x, -c3_tw32[12].y));  // w^3
                const float2 o5 = cmul(y[5], make_float2(c3_tw32[20].x, -c3_tw32[20].y));  // w^5
                const float2 o7 = cmul(y[7], make_float2(c3_tw32[28].x, -c3_tw32[28].y));  // w^7
                const float2 O1 = make_float2(o1.x + o3.x + o5.x + o7.x, o1.y + o3.y + o5.y + o7.y);
                const float2 z0 = make_float2(E0.x + O0.x, E0.y + O0.y);
                const float2 z4 = make_float2(E0.x - O0.x, E0.y - O0.y);
                const float2 z1 = make_float2(E1.x + O1.x, E1.y + O1.y);
                const float2 z5 = make_float2(E1.x - O1.x, E1.y - O1.y);
                const float2 c4 = s_carry[warp][slot][0][k][lane];
                const float2 c5 = s_carry[warp][slot][1][k][lane];
                RA[k] = make_float2(z0.x + c4.x, z0.y + c4.y);
                RB[k] = make_float2(z1.x + c5.x, z1.y + c5.y);
                s_carry[warp][slot][0][k][lane] = z4;
                s_carry[warp][slot][1][k][lane] = z5;
            }
        }

        if (m < m0) continue;   // warm-up step: only the carries are needed

        // Inverse Y: fold ky and ky+16 for each output field's row parity.
        const int j = lane >> 4;
        const int i = lane & 15;
        const int kk = rev4(i);
        const int f = 2 * m + j;
        const int p = f & 1;
        const int y0 = (p - tileY) & 1;
        float2 G[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const float2 send = j ? RA[k] : RB[k];
            const float2 recv = shfl_xor2(send, 16);
            float2 lo_v, hi_v;   // R[kk], R[kk+16] of this half-warp's field
            if (j == 0) { lo_v = RA[k]; hi_v = recv; }
            else { lo_v = recv; hi_v = RB[k]; }
            float2 s = y0 ? make_float2(lo_v.x - hi_v.x, lo_v.y - hi_v.y) : make_float2(lo_v.x + hi_v.x, lo_v.y + hi_v.y);
            // exp(+i pi kk y0 / 16) = conj(tw32[kk]) when y0 = 1
            if (y0) s = cmul(s, make_float2(c3_tw32[kk].x, -c3_tw32[kk].y));
            G[k] = s;
        }
        // 16-point inverse DFT, bit-reversed input -> natural order (DIT)
#pragma unroll
        for (int h = 1; h <= 8; h <<= 1) {
            const bool upper = (i & h) != 0;
            const int r = i & (h - 1);
            const float2 w = make_float2(c3_tw16[r * (8 / h)].x, -c3_tw16[r * (8 / h)].y);   // exp(+2 pi i r/(2h))
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const float2 o = shfl_xor2(G[k], h);
                if (upper) {
                    const float2 t = cmul(G[k], w);
                    G[k] = make_float2(o.x - t.x, o.y - t.y);
                } else {
                    const float2 t = cmul(o, w);
                    G[k] = make_float2(G[k].x + t.x, G[k].y + t.y);
                }
            }
        }
        // Inverse X and store: lane holds row i of field 2m + j.
        const int y = y0 + 2 * i;
        const int L = tileY + y;
        if (L >= P.fafl && L <= P.lafl) {
            float o[16];
#pragma unroll
            for (int x = 0; x < 8; x++) {
                float C = 0.f, S = 0.f;
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    C = __fmaf_rn(G[k].x, c3_cix[k][x], C);
                    S = __fmaf_rn(G[k].y, c3_six[k][x], S);
                }
                o[x] = C - S;
                o[15 - x] = C + S;
            }
            const int ofield = 2 * (m - P.frame_begin) + j;
            float *dst = P.partial + (long long)cls * P.part_class_stride + (long long)ofield * P.part_field_stride +
                         (long long)((L >> 1) - P.fl_lo) * P.part_row_stride - P.avs;
#pragma unroll
            for (int x = 0; x < 16; x++) {
                const int X = tileX + x;
                if (X >= P.avs && X < P.ave) dst[X] = o[x];
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
    float dfx[5][16][4], dfwy[32][2], dfwz[8][2], dftw32[32][4];
    for (int k = 0; k < 5; k++)
        for (int x = 0; x < 16; x++) {
            const double w = rc_window(x, 16);
            const double a = -2.0 * M_PI * (k + 2) * x / 16.0;
            split_df(w * cos(a), dfx[k][x][0], dfx[k][x][1]);
            split_df(w * sin(a), dfx[k][x][2], dfx[k][x][3]);
        }
    for (int y = 0; y < 32; y++) split_df(rc_window(y, 32), dfwy[y][0], dfwy[y][1]);
    for (int z = 0; z < 8; z++) split_df(rc_window(z, 8), dfwz[z][0], dfwz[z][1]);
    for (int r = 0; r < 32; r++) {
        split_df(cos(-2 * M_PI * r / 32), dftw32[r][0], dftw32[r][1]);
        split_df(sin(-2 * M_PI * r / 32), dftw32[r][2], dftw32[r][3]);
    }
#define TPAL_CPY(sym, src)                                                  \
    if (cudaMemcpyToSymbol(sym, src, sizeof(src)) != cudaSuccess) return -1;
    TPAL_CPY(c3_cwx, cwx);
    TPAL_CPY(c3_swx, swx);
    TPAL_CPY(c3_cix, cix);
    TPAL_CPY(c3_six, six);
    TPAL_CPY(c3_wy, wy);
    TPAL_CPY(c3_wx, wx);
    TPAL_CPY(c3_wz, wz);
    TPAL_CPY(c3_tw16, tw16);
    TPAL_CPY(c3_tw32, tw32);
    TPAL_CPY(c3_dfx, dfx);
    TPAL_CPY(c3_dfwy, dfwy);
    TPAL_CPY(c3_dfwz, dfwz);
    TPAL_CPY(c3_dftw32, dftw32);
#undef TPAL_CPY
    if (device >= 0 && device < 64) g_tp3_constants_ready[device] = true;
    return 0;
}

int tp3_launch(const T3Params &P, cudaStream_t stream)
{
    const long long items = (long long)P.ntx * P.nty * P.nchunks;
    if (items <= 0) return 0;
    const unsigned blocks = (unsigned)((items + kWarps3 - 1) / kWarps3);
    tpal3d_kernel<<<blocks, 32 * kWarps3, 0, stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace tpal
