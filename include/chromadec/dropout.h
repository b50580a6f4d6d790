/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Dropout concealment and detection queries (reference:
 * include/chromadec/dropout.h). Concealment runs on the GPU, bit-exact with
 * the reference's single-source DropoutCorrector. */
#ifndef CHROMADEC_DROPOUT_H
#define CHROMADEC_DROPOUT_H

#include <chromadec/enum.h>
#include <chromadec/errors.h>
#include <chromadec/types.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct chd_dropout_opts {
    int enabled;
    int overcorrect;        /* extend dropout boundaries by +-24 samples */
    int intra_field_only;   /* skip cross-field replacement candidates */
    void *reserved[4];
} chd_dropout_opts_t;

typedef struct chd_dropout_stats {
    int32_t corrected;
    int32_t failed;
    int64_t total_distance;
} chd_dropout_stats_t;

chd_status_t chd_decoder_set_dropout(chd_decoder_t *d, const chd_dropout_opts_t *opts);   /* dropout.h:30 */
chd_status_t chd_decoder_get_last_dropout_stats(const chd_decoder_t *d, chd_dropout_stats_t *out); /* :33-34 */

typedef CHD_ENUM(chd_dropout_origin) {
    CHD_DROPOUT_ORIGIN_SOURCE_METADATA     = 0,
    CHD_DROPOUT_ORIGIN_DECODER_CONCEALMENT = 8
} chd_dropout_origin_t;

/* A run of dropped samples on one output row: x in [x_start, x_end). */
typedef struct chd_dropout_span {
    int32_t y;
    int32_t x_start;
    int32_t x_end;
    chd_dropout_origin_t origin;
} chd_dropout_span_t;

typedef CHD_ENUM(chd_dropout_detect_mode) {
    CHD_DROPOUT_DETECTED    = 0,
    CHD_DROPOUT_OVERCORRECT = 1
} chd_dropout_detect_mode_t;

/* Spans of one frame in output framing, sorted by (y, x_start); free with
 * chd_dropout_spans_free (reference dropout.h:67-73). */
chd_status_t chd_decoder_get_dropout_spans(chd_decoder_t *d, int64_t frame_index, chd_dropout_detect_mode_t mode,
                                           chd_dropout_span_t **out_spans, size_t *out_count);
void chd_dropout_spans_free(chd_dropout_span_t *spans);

/* The spans rasterised into a one-plane GRAY16 (0xFFFF) or GRAYS (1.0) mask
 * frame (reference dropout.h:82-85). */
chd_status_t chd_decode_dropout_mask(chd_decoder_t *d, int64_t frame_index, chd_dropout_detect_mode_t mode,
                                     chd_frame_t **out);

#ifdef __cplusplus
}
#endif
#endif
