// tpal_kernels.h -- launch parameters of the sm_103a kernels (host + device).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tpal {

// Device field buffer: field f (absolute index in the capture, first field of
// each frame at even f) starts at fields + (f - field_base) * field_stride;
// the buffer holds every capture field the launch reads. Fields outside
// [0, nfields) are black padding frames and read as zero after black removal.
//
// Chroma partial planes: 4 overlap classes x output fields x rows x cols, in
// FP32; row r is field line fl_lo + r, column c is sample avs + c. Output
// field o is field 2 * frame_begin + o.

// Field f's first sample: from the batch table when there is one (null for
// a black field), else field f of the contiguous buffer.
template <typename Params>
__device__ __forceinline__ const uint16_t *field_at(const Params &P, int f)
{
    if (P.field_ptrs != nullptr) return P.field_ptrs[f];
    return P.fields + (long long)(f - P.field_base) * P.field_stride;
}

// Deferred exact decisions of the 3D transform. The walk decides every bin
// in FP32 and, for each kx group with a bin inside the guard band, appends
// one record; the resolve pass decides those bins exactly and lists the work
// items where FP32 got one wrong, which the exact walk then runs again with
// every guard-band decision taken exactly, overwriting their output.
struct UncRecord {
    int item;            // work item (tile + ntiles * chunk)
    int tile;            // tile position, tx + ntx * ty
    int m;               // the Z tile T(2m)
    int g;               // kx group: column A is kx = 2 + g
    uint8_t unc[32];     // per lane (ky = kappa(lane)): kz bits inside the guard band
    uint8_t keep[32];    // per lane: the FP32 decisions the walk used
};

struct T3Params {
    const uint16_t *fields;      // buffer holding fields [field_base, ...)
    const uint16_t *const *field_ptrs;   // or (batches) each field's first sample by index, null = black
    long long field_stride;
    int field_base;
    int nfields;
    int fw, fh;                  // samples per line, lines per field
    int avs, ave, fafl, lafl;   // active samples [avs, ave), frame lines [fafl, lafl]
    int black;
    int swap;                    // 1: even fields are second fields (reversed pairing)
    int tileX0, ntx, tileY0, nty;
    int frame_begin, frame_end, chunk_frames, nchunks;
    float *partial;
    long long part_class_stride, part_field_stride;
    int part_row_stride, fl_lo;
    float t2f, t2hi, t2lo;       // uniform squared threshold (FP32 and double-float)
    const float *thr_table;      // per-bin squared thresholds [8][32][3] x (f, hi, lo), or null
    const float *frame_t2;       // per-frame squared threshold (f, hi, lo) by frame index, or null (batches)
    unsigned int *stats;         // [0] exact decisions taken, [1] of which FP32 was wrong
    // deferred exact decisions (required)
    UncRecord *unc_rec;
    unsigned int *rerun;         // (work item, step) pairs to walk again exactly (unc_cap pairs)
    unsigned int *counters;      // [0] records, [1] items listed in rerun
    unsigned int unc_cap;
};

struct T2Params {
    const uint16_t *fields;
    const uint16_t *const *field_ptrs;   // or (batches) each field's first sample by index, null = black
    long long field_stride;
    int field_base;
    int nfields;
    int fw;
    int avs, ave, fafl, lafl;
    int black;
    int swap;                    // 1: even fields are second fields (reversed pairing)
    int field_begin, nout;       // output fields [field_begin, field_begin + nout)
    float *partial;
    long long part_class_stride, part_field_stride;
    int part_row_stride, fl_lo;
    float t2f, t2hi, t2lo;
    const float *thr_table;      // [16][5] x (f, hi, lo), or null
    const float *frame_t2;       // per-frame squared threshold (f, hi, lo) by frame index, or null (batches)
    unsigned int *stats;
};

// PALcolour demodulation + H.273 pack of output fields.
struct DemodParams {
    const uint16_t *fields;      // same buffer as the transform's
    const uint16_t *const *field_ptrs;   // or (batches) each field's first sample by index, null = black
    long long field_stride;
    int field_base;
    int field_begin, nout;       // output field o is absolute field field_begin + o
    int fw, fh;
    int avs, ave, fafl, lafl;
    int burst_start, burst_end;
    int black, white;
    const float *partial;        // chroma partial planes as above (NULL: demodulate the composite)
    long long part_class_stride, part_field_stride;
    int part_row_stride, fl_lo;
    int nclasses;                // 4 for the Transform kinds
    int swap;                    // 1: even window fields are second fields (offset = (f & 1) ^ swap)
    float gain_cos, gain_sin;    // chroma_gain * (cos, sin)(chroma_phase)
    float nr_y;                  // luma coring level in sample units (0 = off)
    int format;                  // chd_pixel_format_t: 0 yuv444p16, 1 yuv444ps, 2 rgb48, 3 rgbs, 4 gray16, 5 grays
    void *out;                   // frames in the format's layout, out_w x out_h
    void *const *frame_out;      // per-frame output pointers by frame index (null entry: not written), or null
    long long out_frame_stride;  // elements per frame
    int out_w, out_h, left_pad, top_pad;
    float ey_scale, ecb_scale, ecr_scale;   // 1/range, ecbFromU/range, ecrFromV/range
    // the integer formats' code scales, each split hi + lo from double:
    // 219*256/range (Y, gray16), 224*256*ecbFromU/range, 224*256*ecrFromV/range
    float qy_hi, qy_lo, qcb_hi, qcb_lo, qcr_hi, qcr_lo;
    float y_lo, y_hi, c_lo, c_hi;           // Y'CbCr clamp bounds (code units for p16/gray16, E' for ps/grays)
    float rgb_y_scale, rgb_uv_scale;        // rgb48: 65535/range; rgbs: 1/range
    float r_from_v, g_from_u, g_from_v, b_from_u;
    float r_lo, r_hi, g_lo, g_hi, b_lo, b_hi;   // R'G'B' clamp bounds
    float cfilt[8][4];           // chroma FIR taps of the sample rate (PalColour::buildLookUpTables)
    float yfilt[8][2];           // luma-extraction taps
    int swap_carrier;            // 1 at fieldHeight 263: the reference's PAL-M sine/cosine exchange
};

// Learned-mask form of the 3D transform: the walk's two extra passes.
// Per Z tile T(2m) (zi = m - z0) and spatial tile, the 1,280 bins the filter
// can keep are indexed v = (q * 8 + kz) * 32 + ky with q = kx - 2 in 0..4.
struct T3Learn {
    // feature pass (learned_pass 0): outputs, each [nz][ntiles][1280]
    uint16_t *feat;              // bf16 bits of ln(1 + |X|) / 16
    float2 *spec;                // the complex spectrum X (optional)
    float *plain_p;              // the FP32 threshold decisions as 0 / 1 (optional)
    // apply pass (learned_pass 1): inputs
    const float *p;              // kept fraction of each bin [nz][ntiles][1280]
    const uint8_t *fallback;     // [nz][ntiles]: 1 = the tile takes the threshold decisions instead
    int z0;                      // Z tile index of step m: m - z0
};

int tp3_init_constants(int device);
// max_blocks > 0 caps the grid; the blocks then walk the work items persistently.
int tp3_launch(const T3Params &p, cudaStream_t stream, int max_blocks = 0);
// The resolve pass and the exact walk of the listed items (after
// tp3_launch; the counters are zeroed before it).
int tp3_resolve_launch(const T3Params &p, cudaStream_t stream);
// Learned form: pass 0 writes the features (and optionally the spectrum and
// the FP32 threshold decisions) of every Z tile of frames
// [frame_begin, frame_end)'s walk; pass 1 walks again applying the fractions
// and writes the overlap-class planes. Uniform threshold only.
int tp3_learned_launch(const T3Params &p, const T3Learn &l, int pass, cudaStream_t stream);
// Records one launch can write at most: every kx group of every step.
constexpr unsigned long long tp3_unc_capacity(int ntiles, int frames, int nchunks)
{
    return (unsigned long long)ntiles * (unsigned long long)(frames + 2 * nchunks) * 3ull;
}
int tp2_init_constants(int device);
int tp2_launch(const T2Params &p, cudaStream_t stream);
// Tensor-core form of the 3D transform stage (tc3d.cu): the same overlap-class
// planes as tp3_launch, with the DFT stages as split-precision tcgen05
// contractions (variant 0 = 3xTF32, 1 = BF16x3) and FP32 decisions on their
// spectra. Uniform threshold, one capture buffer.
int tc3_transform(const T3Params &p, int field_height, int variant, cudaStream_t stream);
int tc3_launches_per_frames(int frames);
int demod_init_constants(int device);
int demod_taps(double sample_rate, float (&cfilt)[8][4], float (&yfilt)[8][2]);
int demod_launch(const DemodParams &p, cudaStream_t stream);

}  // namespace tpal
