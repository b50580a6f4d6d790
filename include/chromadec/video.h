/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Library lifecycle and composite sources of the chd_* ABI
 * (reference: include/chromadec/video.h). */
#ifndef CHROMADEC_VIDEO_H
#define CHROMADEC_VIDEO_H

#include <chromadec/errors.h>
#include <chromadec/types.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces reference video.h:12-13. */
chd_status_t chd_init(void);
void         chd_shutdown(void);

/* Open an ld-decode `.tbc` capture (uint16 fields) with its JSON sidecar:
 * metadata_path_or_null = NULL looks for `<path>.json`. PAL / PAL-M
 * line-locked captures decode on the GPU; other sidecars open and report
 * their geometry. Replaces reference video.h:31-34. */
chd_status_t chd_video_open_composite(const char *path,
                                      const char *metadata_path_or_null,
                                      const chd_video_params_t *override_or_null,
                                      chd_video_t **out);

/* Dual-file Y/C captures are not on the Transform-PAL path:
 * CHD_E_UNSUPPORTED. Replaces reference video.h:42-46. */
chd_status_t chd_video_open_yc(const char *luma_path, const char *chroma_path,
                               const char *metadata_path_or_null,
                               const chd_video_params_t *override_or_null,
                               chd_video_t **out);

void         chd_video_free(chd_video_t *v);                         /* reference video.h:48 */
chd_status_t chd_video_get_info(const chd_video_t *v, chd_video_info_t *out);   /* reference video.h:50 */

/* Woven frame line <-> field-sequential signal line (reference video.h:80-83). */
chd_status_t chd_video_frame_line_to_signal_line(const chd_video_t *v, int32_t frame_line, int32_t *out);
chd_status_t chd_video_signal_line_to_frame_line(const chd_video_t *v, int32_t signal_line, int32_t *out);

/* Row sample <-> interface-standard sample (reference video.h:109-112). */
chd_status_t chd_video_standard_sample_to_row_sample(const chd_video_t *v, int32_t standard_sample,
                                                     int32_t *out);
chd_status_t chd_video_row_sample_to_standard_sample(const chd_video_t *v, int32_t row_sample, int32_t *out);

/* Multi-source dropout correction needs extra captures and VBI alignment,
 * outside this path: CHD_E_UNSUPPORTED. Replaces reference video.h:116-122. */
chd_status_t chd_video_add_extra_source_composite(chd_video_t *v, const char *path,
                                                  const char *metadata_path_or_null);
chd_status_t chd_video_add_extra_source_yc(chd_video_t *v, const char *luma_path, const char *chroma_path,
                                           const char *metadata_path_or_null);

#ifdef __cplusplus
}
#endif
#endif
