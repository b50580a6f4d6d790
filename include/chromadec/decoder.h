/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Decoder handles, options, commit and decode of the chd_* ABI
 * (reference: include/chromadec/decoder.h). CHD_DEC_TRANSFORM_2D and
 * CHD_DEC_TRANSFORM_3D decode on the GPU; every other kind is accepted at
 * create/option time exactly like the reference and rejected at commit with
 * CHD_E_UNSUPPORTED. */
#ifndef CHROMADEC_DECODER_H
#define CHROMADEC_DECODER_H

#include <chromadec/enum.h>
#include <chromadec/errors.h>
#include <chromadec/types.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Values of the reference's decoder.h:14-33. */
typedef CHD_ENUM(chd_decoder_kind) {
    CHD_DEC_AUTO                  = 0,
    CHD_DEC_MONO                  = 1,
    CHD_DEC_NTSC_1D               = 2,
    CHD_DEC_NTSC_2D               = 3,
    CHD_DEC_NTSC_3D               = 4,
    CHD_DEC_NTSC_3D_NO_ADAPT      = 5,
    CHD_DEC_PAL_2D                = 6,
    CHD_DEC_TRANSFORM_2D          = 7,
    CHD_DEC_TRANSFORM_3D          = 8,
    CHD_DEC_NN_TRANSFORM3D        = 9,
    CHD_DEC_LDZEUG_COLOR_CNN      = 10,
    CHD_DEC_LDZEUG_LUMA_SEP       = 11,
    CHD_DEC_LDZEUG_LUMA_SEP_FRAME = 12,
    CHD_DEC_NONE                  = 13,
    CHD_DEC_SECAM                 = 20,
    CHD_DEC_HVD_2D                = 30,
    CHD_DEC_HVD_3D                = 31
} chd_decoder_kind_t;

chd_status_t chd_decoder_create(chd_video_t *v, chd_decoder_kind_t kind, chd_decoder_t **out);  /* decoder.h:35 */
void         chd_decoder_free(chd_decoder_t *d);                                                 /* decoder.h:36 */

/* Typed option setters; CHD_E_INVALID_ARG for an option that does not apply
 * to the kind or after commit (reference decoder.h:40-44). */
chd_status_t chd_decoder_set_option_f64(chd_decoder_t *d, const char *name, double v);
chd_status_t chd_decoder_set_option_i32(chd_decoder_t *d, const char *name, int32_t v);
chd_status_t chd_decoder_set_option_bool(chd_decoder_t *d, const char *name, int v);
chd_status_t chd_decoder_set_option_str(chd_decoder_t *d, const char *name, const char *v);
chd_status_t chd_decoder_has_option(const chd_decoder_t *d, const char *name);

/* No NN decoder kinds here (reference decoder.h:46; the reference returns
 * the same status when built without NN support). */
chd_status_t chd_decoder_set_nn_model(chd_decoder_t *d, chd_nn_model_t *m);

/* Apply pending options; idempotent (reference decoder.h:49). */
chd_status_t chd_decoder_commit(chd_decoder_t *d);

/* Committed output framing (reference decoder.h:55). */
chd_status_t chd_decoder_get_output_info(const chd_decoder_t *d, chd_output_info_t *out);

#define CHD_OPT_CHROMA_GAIN                 "chroma_gain"
#define CHD_OPT_CHROMA_PHASE_DEG            "chroma_phase_deg"
#define CHD_OPT_CHROMA_NR_LEVEL             "chroma_nr_level"
#define CHD_OPT_LUMA_NR_LEVEL               "luma_nr_level"
#define CHD_OPT_PADDING_MULTIPLE            "padding_multiple"
#define CHD_OPT_REVERSE_FIELD_ORDER         "reverse_field_order"
#define CHD_OPT_PHASE_COMPENSATION          "phase_compensation"
#define CHD_OPT_COMB_ADAPT_THRESHOLD        "comb_adapt_threshold"
#define CHD_OPT_COMB_CHROMA_WEIGHT          "comb_chroma_weight"
#define CHD_OPT_COMB_SHOW_MAP               "comb_show_map"
#define CHD_OPT_CHROMA_IDENT_MODE           "chroma_ident_mode"
#define CHD_OPT_CHROMA_IDENT_MANUAL         "chroma_ident_manual"
#define CHD_OPT_CHROMA_CLICK_NR_LEVEL       "chroma_click_nr_level"
#define CHD_OPT_CHROMA_CLICK_ENV_DIP_DB     "chroma_click_env_dip_db"
#define CHD_OPT_CHROMA_CLICK_FREQ_OVERSHOOT "chroma_click_freq_overshoot"
#define CHD_OPT_TRANSFORM_THRESHOLD         "transform_threshold"
#define CHD_OPT_TRANSFORM_THRESHOLDS_FILE   "transform_thresholds_file"
#define CHD_OPT_FIRST_ACTIVE_SAMPLE         "first_active_sample"
#define CHD_OPT_LAST_ACTIVE_SAMPLE          "last_active_sample"
#define CHD_OPT_FIRST_ACTIVE_FRAME_LINE     "first_active_frame_line"
#define CHD_OPT_LAST_ACTIVE_FRAME_LINE      "last_active_frame_line"
#define CHD_OPT_NN_INPUT_MAGNITUDE_SCALE    "nn_input_magnitude_scale"
#define CHD_OPT_NN_CHROMA_BANDPASS          "nn_chroma_bandpass"
#define CHD_OPT_HVD_CG_ITERATIONS           "hvd_cg_iterations"
#define CHD_OPT_HVD_TEMPORAL_STRENGTH       "hvd_temporal_strength"
#define CHD_OPT_OUTPUT_FORMAT               "output_format"
#define CHD_OPT_OUTPUT_CLAMP                "output_clamp"
#define CHD_OPT_COLOR_DIFFERENCE_PRECISION  "color_difference_precision"
#define CHD_OPT_BROADCAST_SCALING_PRECISION "broadcast_scaling_precision"
#define CHD_OPT_OUTPUT_Y4M_HEADERS          "output_y4m_headers"
#define CHD_OPT_THREAD_COUNT                "thread_count"

/* SECAM-only query (reference decoder.h:92-94): CHD_E_UNSUPPORTED here. */
chd_status_t chd_decoder_get_chroma_click_thresholds(const chd_decoder_t *d, double *env_dip_db,
                                                     double *freq_overshoot);

/* Decode one frame (reference decoder.h:98). Consecutive requests are
 * decoded ahead in batches on the GPU and returned one at a time. */
chd_status_t chd_decode_frame(chd_decoder_t *d, int64_t frame_index, chd_frame_t **out);

/* Decode many frames; cb receives each (status, index, frame) in completion
 * order and owns the frame. Blocks until every index has been delivered
 * (reference decoder.h:100-104). */
typedef void (*chd_frame_done_cb)(void *user, chd_status_t s, int64_t idx, chd_frame_t *f);
chd_status_t chd_decode_frames_async(chd_decoder_t *d, const int64_t *indices, size_t n, chd_frame_done_cb cb,
                                     void *user, chd_cancel_t *cancel_or_null);

#ifdef __cplusplus
}
#endif
#endif
