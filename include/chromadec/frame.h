/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Decoded frames (reference: include/chromadec/frame.h). Planes are borrowed:
 * valid until chd_frame_free, which the caller owns. */
#ifndef CHROMADEC_FRAME_H
#define CHROMADEC_FRAME_H

#include <chromadec/errors.h>
#include <chromadec/types.h>

#ifdef __cplusplus
extern "C" {
#endif

chd_status_t chd_frame_get_info(const chd_frame_t *f, chd_frame_info_t *out);                   /* frame.h:12 */
chd_status_t chd_frame_get_plane_info(const chd_frame_t *f, chd_plane_t p, chd_plane_info_t *out); /* frame.h:17 */
/* 4:4:0 (SECAM) only in the reference: CHD_E_UNSUPPORTED for these formats (frame.h:25-31). */
chd_status_t chd_frame_chroma_row_component(const chd_frame_t *f, int32_t frame_row,
                                            chd_chroma_row_component_t *out);
chd_status_t chd_frame_get_chroma_ident(const chd_frame_t *f, chd_chroma_ident_report_t *out);
/* 16-bit planes: yuv444p16 is [Y | Cb | Cr], stride width*2 bytes (frame.h:36-38). */
chd_status_t chd_frame_get_plane(const chd_frame_t *f, chd_plane_t p, const void **out_data,
                                 ptrdiff_t *out_stride_bytes);
/* float planes: yuv444ps E'Y / E'Cb / E'Cr, grays E'Y (frame.h:51-53). */
chd_status_t chd_frame_get_plane_float(const chd_frame_t *f, chd_plane_t p, const float **out_data,
                                       ptrdiff_t *out_stride_bytes);
void chd_frame_free(chd_frame_t *f);                                                             /* frame.h:55 */

#ifdef __cplusplus
}
#endif
#endif
