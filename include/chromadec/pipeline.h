/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Cancellation handles for chd_decode_frames_async (reference:
 * include/chromadec/pipeline.h:17-20). */
#ifndef CHROMADEC_PIPELINE_H
#define CHROMADEC_PIPELINE_H

#include <chromadec/errors.h>
#include <chromadec/types.h>

#ifdef __cplusplus
extern "C" {
#endif

chd_status_t chd_cancel_create(chd_cancel_t **out);
void         chd_cancel_request(chd_cancel_t *c);
int          chd_cancel_is_requested(const chd_cancel_t *c);
void         chd_cancel_free(chd_cancel_t *c);

#ifdef __cplusplus
}
#endif
#endif
