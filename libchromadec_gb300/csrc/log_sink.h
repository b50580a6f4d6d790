// log_sink.h -- the process-wide diagnostics sink behind chd_set_log_callback
// (include/chromadec/log.h; reference: src/common/log.cpp).
#pragma once

#include <chromadec/log.h>

namespace chdg {

// Deliver `message` to the installed sink when `level` passes the threshold.
void log_emit(chd_log_level_t level, chd_log_flags_t flags, const char *message);
// A message that duplicates a failure returned to the caller.
inline void log_returned(chd_log_level_t level, const char *message) { log_emit(level, CHD_LOG_F_RETURNED, message); }

}  // namespace chdg
