/* SPDX-License-Identifier: GPL-3.0-or-later */
/*
 * chromadec_gb300.h -- device-level entry points of libchromadec_gb300.
 *
 * These calls have no counterpart in the reference's public ABI: they expose
 * the GB300 Transform-PAL pipeline on device-resident buffers (CUDA device
 * pointers, a cudaStream_t passed as void*), for callers that already keep
 * captures in HBM and for the benchmark's device-resident measurement. The
 * reference-compatible chd_* ABI in <chromadec/*.h> is built on top of them.
 *
 * Conventions: a capture is a device array of uint16 fields, field f at
 * fields + f * field_stride samples, frame k made of fields 2k and 2k+1 (the
 * first field at the even index unless first_field_offset says otherwise). Frames outside the capture are black padding, as in the reference's
 * SourceField::loadFields (src/decoders/source_field.cpp:88-170). Every call
 * returns 0 on success and a negative CHDG_E_* code on failure; failures
 * also set the thread's chd_last_error() detail.
 */
#ifndef CHROMADEC_GB300_H
#define CHROMADEC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHDG_E_INVALID_ARG  (-1)
#define CHDG_E_UNSUPPORTED  (-2)
#define CHDG_E_CUDA         (-3)
#define CHDG_E_OOM          (-4)

/* Source geometry and levels (the VideoParameters fields the path reads). */
typedef struct chdg_geometry {
    int32_t field_width, field_height;
    int32_t active_start, active_end;                      /* samples, half-open */
    int32_t first_active_frame_line, last_active_frame_line; /* inclusive */
    int32_t burst_start, burst_end;
    int32_t black, white;
    double sample_rate, fsc;
} chdg_geometry;

/* Decoder + output settings (PalColour::Configuration and
 * OutputWriter::Configuration fields the path reads). */
typedef struct chdg_config {
    int32_t kind;                 /* 6 = CHD_DEC_PAL_2D, 7 = CHD_DEC_TRANSFORM_2D, 8 = CHD_DEC_TRANSFORM_3D */
    double threshold;             /* transform_threshold, default 0.4 */
    const double *thresholds;     /* per-bin thresholds (80 for 2D, 768 for 3D) or NULL */
    int32_t n_thresholds;
    double chroma_gain, chroma_phase_deg;
    int32_t output_format;        /* chd_pixel_format_t: 0 yuv444p16, 1 yuv444ps, 2 rgb48, 3 rgbs, 4 gray16, 5 grays */
    int32_t clamp_mode;           /* chd_clamp_t */
    int32_t padding_multiple;     /* 1 = none */
    double ecb_from_u, ecr_from_v;
    /* ColorConversion inputs (src/common/color_conversion.cpp:33-66): luma
     * coefficients and the composite U/V reductions, for the RGB formats */
    double kr, kb, u_reduction, v_reduction;
    double y_nr_level;            /* luma_nr_level (doYNR); 0 = off */
    int32_t first_field_offset;   /* 1: field 2k of every frame is its second field (reverse_field_order) */
} chdg_config;

typedef struct chdg_engine chdg_engine;

/* Fill g with the reference's line-locked 4fsc PAL preset and c with the
 * decoder defaults for `kind` (6, 7 or 8). */
void chdg_default_geometry(chdg_geometry *g);
void chdg_default_config(chdg_config *c, int32_t kind);

/* Create an engine on the current CUDA device. Constant tables are uploaded
 * once per device; scratch grows on demand. The scratch (chroma planes,
 * decision records) is shared by all of an engine's calls: issue them on one
 * stream, or order them with events; decode concurrently with one engine per
 * stream. */
int chdg_engine_create(const chdg_geometry *g, const chdg_config *c, chdg_engine **out);
void chdg_engine_free(chdg_engine *e);

/* Output frame geometry (after padding) and bytes per output frame. */
int chdg_output_geometry(const chdg_engine *e, int32_t *width, int32_t *height, size_t *frame_bytes);

/* Frames per GPU batch of chdg_decode_device (default 256, at least 1): a
 * longer range is decoded in batches of this many frames, with identical
 * results. It bounds the engine's scratch, which grows with the batch: the
 * four chroma planes take about 8.7 MB per frame, and the learned form's
 * tile features, fractions and flags about 34 MB more. */
int chdg_engine_set_max_batch_frames(chdg_engine *e, int32_t frames);

/* Decode frames [frame_begin, frame_end) of a device-resident capture of
 * nfields fields into d_out (frame_end - frame_begin frames, each in the
 * output format's layout: [Y | Cb | Cr] or [R | G | B] planes, interleaved
 * R'G'B' for rgb48, one plane for the gray formats).
 * Asynchronous on `stream`. */
int chdg_decode_device(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                       int32_t frame_begin, int32_t frame_end, void *d_out, void *stream);

/* Decode frames [frame_begin, frame_end) of a capture held in HOST memory
 * (nfields fields, field f at h_fields + f * field_stride samples) into
 * h_out. Field windows are uploaded and frames downloaded in a double-buffered
 * pipeline that overlaps the copies with the kernels (batches of 64 frames, 16
 * at either end of a longer run); use pinned memory for full-rate copies.
 * Completes asynchronously on `stream`; a later call on the same engine
 * reuses its device buffers only after this call's work on them. */
int chdg_decode_host(chdg_engine *e, const uint16_t *h_fields, int64_t field_stride, int32_t nfields,
                     int32_t frame_begin, int32_t frame_end, void *h_out, void *stream);

/* Per-kernel timing of the engine's launches (CUDA events on the launching
 * stream): enable, run, then read the accumulated transform and demodulator
 * milliseconds and the number of kernel launches. */
int chdg_engine_set_profiling(chdg_engine *e, int on);
int chdg_engine_kernel_times(chdg_engine *e, double *ms_transform, double *ms_demod, int64_t *launches);

/* Transform-PAL chroma only: the separated chroma of fields
 * [2*frame_begin, 2*frame_end) as FP32 planes of (last-first field line + 1)
 * rows x (active_end - active_start) columns, rows starting at field line
 * first_active_frame_line / 2. For checking the transform in isolation. */
int chdg_chroma_device(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                       int32_t frame_begin, int32_t frame_end, float *d_chroma, void *stream);

/* Allocation-free Transform-PAL 3D decode (no counterpart in the reference).
 *
 * Same result as chdg_decode_device for kind 8, for callers that cannot
 * allocate device memory while decoding: hosts whose device memory belongs to
 * their own allocator or budget, and latency-critical loops where cudaMalloc's
 * implicit device synchronisation would stall other work. The chroma scratch
 * and the guard-band decision records are fixed arrays compiled into the
 * library (81.6 MB: 8 frames of the 948x576 active picture), which every GPU
 * that loads the library holds until the process exits; calls asking for
 * more than 8 frames, a negative or reversed frame range, or a larger active
 * picture fail with CHDG_E_INVALID_ARG. No cudaMalloc/cudaFree or other
 * allocating call is made. All calls on a device share the one scratch array
 * (it keeps the last call's contents), so calls whose work overlaps on the GPU
 * race: serialise them on one stream. The first call on a device resolves the
 * array's device address and uploads constant tables; make that first call
 * before starting any stream capture. Per-bin thresholds, when given, are
 * copied from pageable host memory into a second static array on `stream`
 * at every call, ordered after the decodes already queued on that stream; a
 * copy from pageable memory cannot be recorded into a graph, so calls with
 * per-bin thresholds cannot be stream-captured. */
int chdg_decode_device_static(const chdg_geometry *g, const chdg_config *c, const uint16_t *d_fields,
                              int64_t field_stride, int32_t nfields, int32_t frame_begin, int32_t frame_end,
                              void *d_out, void *stream);

/* Batches of captures (no counterpart in the reference, which decodes one
 * capture per decoder). Many captures of uneven length and mixed
 * Transform-PAL 2D/3D modes, each with its own threshold, are decoded by one
 * transform and one demodulator launch per mode, reading every capture's
 * fields in place through a table of field pointers: the 3D captures share
 * one frame index space in which 3 black frames separate neighbours -- the
 * black the reference pads every window with -- so every frame equals the
 * single-capture decode. The first decode of a batch shape runs eagerly,
 * the second captures its launches into a CUDA graph, and later
 * decodes of the same captures (same pointers and sizes) replay the graph
 * with one launch. chdg_batch_autotune times the schedule candidates on the
 * caller's batch and keeps the fastest. Captures and outputs are device
 * buffers; the configuration's output format applies to every capture
 * (padding_multiple 1, no per-bin thresholds). Asynchronous on `stream`;
 * graphs need a created stream (on the legacy default stream, NULL, every
 * decode runs eagerly). */
typedef struct chdg_dropout {
    int32_t field;                /* 0-based field of the capture */
    int32_t startx, endx;         /* samples [startx, endx) */
    int32_t field_line;           /* 1-based field line, as ld-decode's metadata counts */
} chdg_dropout;

#define CHDG_CONCEAL 1                /* conceal the capture's dropouts before decoding */
#define CHDG_CONCEAL_OVERCORRECT 2    /* chd_dropout_opts_t.overcorrect */
#define CHDG_CONCEAL_INTRA 4          /* chd_dropout_opts_t.intra_field */

typedef struct chdg_capture {
    const uint16_t *fields;       /* device: field f at fields + f * field_stride */
    int64_t field_stride;
    int32_t nfields;              /* frames = nfields / 2 */
    int32_t kind;                 /* 7 = Transform 2D, 8 = Transform 3D */
    double threshold;             /* transform_threshold of this capture */
    void *out;                    /* device: nfields / 2 output frames */
    /* The capture's dropouts (host array, ld-decode sidecar spans; read when
     * the batch's shape changes, so it must not change between decodes of
     * one batch) and what to do with them: `conceal` = CHDG_CONCEAL (plus
     * _OVERCORRECT / _INTRA) conceals them as DropoutCorrector does
     * (src/dropout/dropout_corrector.cpp:50-530) on a device copy of the
     * capture -- the caller's fields are not modified -- before decoding;
     * mask_out, when not NULL, receives each frame's dropout mask
     * (chd_decode_dropout_mask's detected mode, GRAY16 0 / 0xFFFF in the
     * output geometry: nfields / 2 planes, device memory). */
    const chdg_dropout *dropouts;
    int32_t ndropouts;
    int32_t conceal;
    uint16_t *mask_out;
} chdg_capture;

typedef struct chdg_batch chdg_batch;

typedef struct chdg_batch_tuning {
    int32_t chunk_frames;         /* frames per 3D work item */
    int32_t max_blocks;           /* 3D grid cap (0 = full grid, else persistent) */
    float ms;                     /* the winner's time for the batch */
} chdg_batch_tuning;

int chdg_batch_create(const chdg_geometry *g, const chdg_config *c, chdg_batch **out);
void chdg_batch_free(chdg_batch *b);
int chdg_batch_decode(chdg_batch *b, const chdg_capture *caps, int32_t n, void *stream);
int chdg_batch_autotune(chdg_batch *b, const chdg_capture *caps, int32_t n, void *stream, chdg_batch_tuning *out);

/* Tensor-core form of the Transform-PAL 3D forward transform (no
 * counterpart in the reference; the precision study beside the plain form,
 * which remains the decoder). The spectra of the reference's 8x32x16 tiles
 * (TransformPal3D::forwardFFTTile, src/decoders/palcolour/
 * transform_pal_3d.cpp:168-202) at the bins the filter reads (kx = 2..6), with
 * the X, Y and Z DFT stages run as tcgen05 tensor-core contractions in split
 * precision: variant CHDG_TC_3XTF32 (TF32 hi/lo operands) or CHDG_TC_BF16X3
 * (BF16 hi/lo), three products per contraction, FP32 accumulation.
 *
 * chdg_tc3d_spectra writes the Z tiles m = m_begin .. m_end-1 (Z tile m holds
 * fields 2m .. 2m+7; fields outside the capture are black) of every spatial
 * tile: d_spec is complex float (re, im) [m_end - m_begin][ntiles][8 kz][5 kx]
 * [32 ky], spatial tiles row-major over tileY = first_active_frame_line - 16
 * + 16 ty and tileX = active_start - 8 + 8 tx, kx = 2 + index. The first
 * field of each frame is at the even index. Asynchronous on `stream`;
 * chdg_tc3d_sync waits for it and reports a tensor-core completion wait that
 * ran out (none is expected). chdg_tc3d_operand copies the host-built image
 * of one coefficient operand (stage 0 = X, 1 = Y, 2 = Z forward, 3 = Z,
 * 4 = Y, 5 = X inverse; split 0 = hi, 1 = lo) in its shared-memory layout
 * and returns its size in bytes. */
#define CHDG_TC_3XTF32 0
#define CHDG_TC_BF16X3 1
int chdg_tc3d_spectra(const chdg_geometry *g, int32_t variant, const uint16_t *d_fields, int64_t field_stride,
                      int32_t nfields, int32_t m_begin, int32_t m_end, void *d_spec, void *stream);
int chdg_tc3d_sync(void *stream);
int chdg_tc3d_operand(int32_t variant, int32_t stage, int32_t y0, int32_t split, void *out, size_t bytes);

/* Decode with the tensor-core form: a Transform 3D engine with a uniform
 * threshold runs its transform stage as tcgen05 contractions in `variant`
 * (CHDG_TC_3XTF32 or CHDG_TC_BF16X3) -- forward X/Y/Z, the threshold decision
 * of each visited bin taken in FP32 on those spectra (not re-decided exactly,
 * unlike the plain form), inverse Z/Y/X and overlap-add -- then the same
 * demodulator; -1 restores the plain form. Its scratch is shared by the
 * device's tensor-core calls: serialise them. Stage images 3..5 of
 * chdg_tc3d_operand are the inverse Z, Y, X coefficients. */
int chdg_engine_set_tc_form(chdg_engine *e, int32_t variant);

/* Learned form of Transform-PAL 3D (no counterpart in the reference, which
 * decides every bin by the fixed mirror threshold of
 * TransformPal3D::applyFilter, src/decoders/palcolour/transform_pal_3d.cpp:
 * 249-333; its NTSC nnTransform3D decoder, src/decoders/nntransform3d/
 * nntransform3d_pipeline_cuda.cu:160-244, is the precedent for a learned
 * per-bin mask). A small 3D convolutional network reads each tile's
 * log-magnitude spectrum over the bins the filter can keep -- kz 0..7,
 * ky 0..31, kx 2..6, v = ((kx - 2) * 8 + kz) * 32 + ky, 1,280 per tile -- as
 * two channels, f = ln(1 + |X|) / 16 at the bin and at its mirror about the
 * carrier, and predicts the fraction p of each bin that is chroma: three
 * 3x3x3 convolutions of 16 channels with ReLU (periodic in kz and ky, zero
 * padded in kx), a sigmoid 1x1x1 head; BF16 weights and activations, FP32
 * accumulation; CHDG_MASKNET_PARAMS FP32 parameters in the order W1[27][2][16],
 * b1[16], W2[27][16][16], b2[16], W3[27][16][16], b3[16], wh[16], bh, tap
 * t = (dz + 1) * 9 + (dy + 1) * 3 + (dkx + 1). A tile whose mean |p - 1/2|
 * is below the confidence limit (default 0.1) takes the threshold decisions
 * instead. Networks are trained on the GPU by these kernels: one call is a
 * batch's forward pass, loss L = sum |p X - C|^2 / sum |X|^2 against the
 * true chroma spectrum C, backward pass and Adam step. */
#define CHDG_MASKNET_PARAMS 14753
#define CHDG_MASKNET_BINS 1280
typedef struct chdg_masknet chdg_masknet;
int chdg_masknet_create(chdg_masknet **out);
void chdg_masknet_free(chdg_masknet *n);
int chdg_masknet_set_weights(chdg_masknet *n, const float *weights, int64_t count);
int chdg_masknet_get_weights(const chdg_masknet *n, float *weights, int64_t count);
int chdg_masknet_set_confidence(chdg_masknet *n, float limit);
/* The network's convolutions run on the tensor cores (tcgen05 implicit
 * GEMMs, the default; on = 1) or on the CUDA cores (on = 0, the cross-check).
 * chdg_masknet_sync waits for `stream` and reports a tensor-core completion
 * wait that ran out (none is expected). */
int chdg_masknet_set_tensor_cores(chdg_masknet *n, int32_t on);
int chdg_masknet_sync(const chdg_masknet *n, void *stream);
/* d_feat: ntiles x 1280 bf16 features (device; 16-byte aligned on the
 * tensor cores, where each tile's features are copied by the TMA bulk
 * engine); d_p: ntiles x 1280 FP32; d_fallback: ntiles bytes (1 = the tile
 * takes the threshold) or NULL. */
int chdg_masknet_forward(const chdg_masknet *n, const uint16_t *d_feat, int64_t ntiles, float *d_p,
                         uint8_t *d_fallback, void *stream);
/* One training step on a batch: d_ac holds per bin (|X|^2, Re(C conj X)) as
 * FP32 pairs, ntiles x 1280. learning_rate 0 computes the loss and gradient
 * only. loss (without its constant sum |C|^2 / sum |X|^2 term) and grad
 * (CHDG_MASKNET_PARAMS floats), when not NULL, are filled after the step
 * completes on `stream`. */
int chdg_masknet_train_step(chdg_masknet *n, const uint16_t *d_feat, const float *d_ac, int64_t ntiles,
                            float learning_rate, double *loss, float *grad, void *stream);
/* Training pairs: per bin (|X|^2, Re(C conj X)) from the composite's spectrum
 * X and the true chroma's C (FP32 complex pairs, nbins each). */
int chdg_masknet_pairs(const float *d_spec_x, const float *d_spec_c, int64_t nbins, float *d_ac, void *stream);

/* The learned form's walk passes on a device-resident capture (the engine's
 * conventions): Z tiles T(2m) for m = frame_begin - 2 .. frame_end - 1, in
 * that order, each over the engine's spatial tiles (chdg_tc3d_spectra's
 * order). chdg_learned_features writes every Z tile's 1,280 features (and,
 * when not NULL, its complex spectrum X as FP32 pairs -- with the horizontal
 * origin at the tile centre, i.e. the reference's r2c bin times
 * exp(i pi kx 15 / 16), which leaves |X| and products C conj X of two such
 * spectra unchanged -- and its FP32 threshold decisions as 0 / 1); chdg_learned_chroma decodes the separated chroma, as
 * chdg_chroma_device does, with the given fractions (and fallback flags)
 * applied in place of the threshold. */
int chdg_learned_features(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                          int32_t frame_begin, int32_t frame_end, uint16_t *d_feat, float *d_spec,
                          float *d_threshold_p, void *stream);
int chdg_learned_chroma(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                        int32_t frame_begin, int32_t frame_end, const float *d_p, const uint8_t *d_fallback,
                        float *d_chroma, void *stream);
/* Decode with the learned form (net != NULL) or the plain form (NULL): a
 * Transform 3D engine with a uniform threshold runs the feature pass, the
 * network and the apply pass in place of its transform stage; the engine
 * borrows the network. chdg_engine_learned_stats reports the tiles decoded
 * and how many fell back to the threshold since the engine was created. */
int chdg_engine_set_masknet(chdg_engine *e, chdg_masknet *net);
int chdg_engine_learned_stats(chdg_engine *e, int64_t *tiles, int64_t *fallback_tiles);

/* Multi-source concealment alignment (MultiSourceAlignment::
 * sourceFrameForPrimaryFrame, src/dropout/multi_source_alignment.cpp:54-71):
 * the 0-based frame of extra source `source` (1 = the first added with
 * chd_video_add_extra_source_*) that holds the same disc frame as the
 * primary's 0-based frame `primary_frame`, matched by CAV picture number or
 * CLV time code when both captures carry them and positionally otherwise;
 * -1 when that source does not hold it. Both captures pair their fields in
 * their own order, swapped when reverse_field_order is non-zero. Returns a
 * chd_status_t (CHD_E_OUT_OF_RANGE for an unknown source). */
struct chd_video;
int chdg_video_source_frame(const struct chd_video *v, int32_t reverse_field_order, int32_t source,
                            int32_t primary_frame, int32_t *out_frame);

/* Dropout concealment as the decoder applies it (no counterpart in the
 * reference ABI, whose DropoutCorrector::correctFrame,
 * src/dropout/dropout_corrector.cpp:50-157, works on the decoder's private
 * field copies): the two fields of frame `frame_index` of a committed
 * decoder, in the decoder's field order (first field first unless
 * reverse_field_order), after the GPU concealment kernel has run that
 * frame's plan with the decoder's current chd_decoder_set_dropout settings
 * and extra sources -- the composite the transform reads. out holds
 * 2 * field_width * field_height uint16 samples. Returns a chd_status_t. */
int chdg_decoder_concealed_fields(struct chd_decoder *d, int64_t frame_index, uint16_t *out);

/* Threshold decisions whose FP32 margin was inside the error bound and were
 * re-evaluated in double-float, and how many of those FP32 had wrong. */
int chdg_engine_stats(chdg_engine *e, uint64_t *exact_decisions, uint64_t *fp32_flips);

#ifdef __cplusplus
}
#endif
#endif
