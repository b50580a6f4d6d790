/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Diagnostics (reference: include/chromadec/log.h:14-71): a process-wide
 * sink, a level threshold (default INFO), and CHD_LOG_F_RETURNED on messages
 * that duplicate a failure returned to the caller. */
#ifndef CHROMADEC_LOG_H
#define CHROMADEC_LOG_H

#include <chromadec/enum.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef CHD_ENUM(chd_log_level) {
    CHD_LOG_DEBUG = 0,
    CHD_LOG_INFO  = 1,
    CHD_LOG_WARN  = 2,
    CHD_LOG_ERROR = 3,
    CHD_LOG_OFF   = 4
} chd_log_level_t;

typedef unsigned int chd_log_flags_t;
#define CHD_LOG_F_RETURNED 0x1u

typedef void (*chd_log_fn)(chd_log_level_t level, chd_log_flags_t flags, const char *message, void *user_data);

void            chd_set_log_callback(chd_log_fn fn_or_null, void *user_data);
void            chd_log_to_stderr(void);
void            chd_set_log_level(chd_log_level_t min_level);
chd_log_level_t chd_get_log_level(void);
int             chd_log_is_enabled(chd_log_level_t level);
const char     *chd_log_level_str(chd_log_level_t level);

#ifdef __cplusplus
}
#endif
#endif
