/*
 * tpal_oracle.h -- CPU oracle for the Transform-PAL hot path.
 *
 * TEST INFRASTRUCTURE, NOT THE PRODUCT. Only the tests, the smoke check and
 * the benchmark's CPU-baseline leg use this library, and only as the checker
 * or as the timed stand-in for the reference's CPU path. The product path
 * (libchromadec_gb300) never links or calls it.
 *
 * It restates, in plain C with FP64 arithmetic and the FP64 DFT of fft64.c,
 * the reference's per-frame Transform-PAL decode:
 *   field window + black padding   src/decoders/source_field.cpp:68-171
 *   TransformPal 2D / 3D           src/decoders/palcolour/transform_pal_2d.cpp:107-287
 *                                  src/decoders/palcolour/transform_pal_3d.cpp:64-333
 *   PALcolour demodulator          src/decoders/palcolour/palcolour.cpp:150-646
 *     (Transform PAL chroma, or the PALcolour 2D filter on the composite,
 *      and the optional luma noise coring doYNR)
 *   second-field shift (scLocked)  src/decoders/source_field.cpp:45-66
 *   output formats                 src/output/output_writer.cpp:52-143,195-239,340-486,670-779
 *   dropout concealment            src/dropout/dropout_corrector.cpp:50-530
 *   dropout spans / mask           src/abi/c_api_dropout_detect.cpp:92-295
 * Operation order follows the reference so results agree to the last bit
 * with the reference compiled against the same FP64 DFT (oracle/Makefile
 * "ref" target, driven by ref_harness.cpp).
 */
#ifndef TPAL_ORACLE_H
#define TPAL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Output formats, numbered as chd_pixel_format_t. */
enum { TPO_FMT_P16 = 0, TPO_FMT_PS = 1, TPO_FMT_RGB48 = 2, TPO_FMT_RGBS = 3, TPO_FMT_GRAY16 = 4, TPO_FMT_GRAYS = 5 };
/* Decoder kinds: 1 = PALcolour 2D filter alone, 2 = Transform PAL 2D, 3 = Transform PAL 3D. */
enum { TPO_CLAMP_NONE = 0, TPO_CLAMP_LEGAL_RGB_SDR = 1, TPO_CLAMP_LEGAL_RGB_HDR = 2, TPO_CLAMP_LEGAL_YCBCR_BT601 = 3 };

typedef struct tpo_params {
    /* geometry (VideoParameters) */
    int32_t field_width, field_height;
    int32_t active_start, active_end;                   /* half-open sample range */
    int32_t first_active_frame_line, last_active_frame_line; /* inclusive */
    int32_t burst_start, burst_end;
    int32_t black, white;
    double sample_rate, fsc;
    int32_t is_pal_m;           /* system PAL_M: the PAL-M luma filter of the dropout corrector (the
                                   demodulator's table swap follows field_height 263, as the reference's) */
    /* decoder */
    int32_t kind;               /* 2 = Transform 2D, 3 = Transform 3D */
    double threshold;
    const double *thresholds;   /* optional per-bin thresholds (not squared), NULL for uniform */
    int32_t n_thresholds;
    double chroma_gain, chroma_phase_deg;
    /* output */
    int32_t output_format;      /* TPO_FMT_* */
    int32_t clamp_mode;         /* TPO_CLAMP_* */
    int32_t padding_multiple;   /* 1 = none */
    double ecb_from_u, ecr_from_v;  /* colour-difference scalars (color_conversion.cpp:59-60) */
    /* ColorConversion inputs for the RGB formats (color_conversion.cpp:33-66) */
    double kr, kb, u_reduction, v_reduction;
    double y_nr_level;          /* luma_nr_level; 0 = off */
    int32_t first_field_offset; /* offset of window slot 0: 0 = first field (normal), 1 = reversed pairing */
    int32_t sc_locked;          /* subcarrier-locked PAL: slot-1 fields shifted left by 2 samples */
} tpo_params;

typedef struct tpo_dropout {
    int32_t field;              /* 0-based field index in the capture */
    int32_t startx, endx;       /* half-open samples */
    int32_t field_line;         /* 1-based */
} tpo_dropout;

/* An extra capture of the same disc for multi-source concealment
 * (chd_video_add_extra_source_composite): its fields in pairing order
 * (frame k = fields 2k (slot 0) and 2k+1 (slot 1)), its dropouts, per-field
 * VITS bPSNR (NULL = 0) and, per primary frame, the frame of this capture
 * that holds the same picture (-1 = not held; frame_map NULL = the same
 * frame index, the reference's positional alignment). */
typedef struct tpo_extra {
    const uint16_t *fields;
    int32_t nfields;
    const struct tpo_dropout *dropouts;
    int32_t ndropouts;
    const double *bpsnr;
    const int32_t *frame_map;
    int32_t nframe_map;
} tpo_extra;

/* The sources of a decode: the primary's per-field bPSNR (NULL = 0) and up
 * to 8 extra captures. */
typedef struct tpo_sources {
    const double *bpsnr;
    const tpo_extra *extras;
    int32_t nextras;
} tpo_sources;

typedef struct tpo_stats {
    int64_t corrected, failed, total_distance;
} tpo_stats;

/* Fill p with the reference's line-locked PAL defaults and decoder defaults. */
void tpo_default_params(tpo_params *p, int32_t kind);

/* Output geometry after padding. */
void tpo_output_geometry(const tpo_params *p, int32_t *width, int32_t *height,
                         int32_t *left_pad, int32_t *top_pad);

/* Bytes of one output frame. */
size_t tpo_frame_bytes(const tpo_params *p);

/* Decode frames [first, first+count) of a capture of nfields fields
 * (field_width*field_height uint16 each, in pairing order: frame k is fields
 * 2k and 2k+1, slot 0 having offset first_field_offset). Dropouts, when
 * given, are concealed before decoding exactly as the reference does.
 * Output: count frames back to back in the output format's layout
 * (OutputFrame / float planes). nthreads >= 1 decodes frames in parallel, one decoder
 * instance per thread (chd_decode_frames_async's model). stats (optional)
 * receives the sum over the decoded frames of their own dropout stats.
 * Returns 0 on success. */
int tpo_decode_frames(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                      const tpo_dropout *dropouts, int32_t ndropouts,
                      int32_t overcorrect, int32_t intra_field,
                      int32_t first, int32_t count, void *out, int32_t nthreads,
                      tpo_stats *stats);

/* tpo_decode_frames with extra sources for multi-source concealment
 * (sources NULL = single source). */
int tpo_decode_frames_ms(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                         const tpo_dropout *dropouts, int32_t ndropouts, const tpo_sources *sources,
                         int32_t overcorrect, int32_t intra_field, int32_t first, int32_t count, void *out,
                         int32_t nthreads, tpo_stats *stats);

/* Transform-PAL chroma (the TransformPal::filterFields output) for the two
 * fields of each frame in [first, first+count): 2*count arrays of
 * field_width*field_height doubles. */
int tpo_transform_chroma(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                         int32_t first, int32_t count, double *out);

/* Conceal the dropouts of frame `frame` and write its two corrected fields
 * (2*field_width*field_height uint16). */
int tpo_dropout_correct_frame(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                              const tpo_dropout *dropouts, int32_t ndropouts,
                              int32_t overcorrect, int32_t intra_field, int32_t frame,
                              uint16_t *out, tpo_stats *stats);

int tpo_dropout_correct_frame_ms(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                                 const tpo_dropout *dropouts, int32_t ndropouts, const tpo_sources *sources,
                                 int32_t overcorrect, int32_t intra_field, int32_t frame, uint16_t *out,
                                 tpo_stats *stats);

typedef struct tpo_span {
    int32_t y, x_start, x_end, origin;
} tpo_span;

/* Dropout spans of frame `frame` in output framing, sorted by (y, x_start);
 * mode 0 = detected, 1 = overcorrect. Returns the number of spans written
 * (at most cap). */
int32_t tpo_dropout_spans(const tpo_params *p, const tpo_dropout *dropouts, int32_t ndropouts,
                          int32_t frame, int32_t mode, tpo_span *out, int32_t cap);

#ifdef __cplusplus
}
#endif
#endif
