// abi_log.cpp -- chd_set_log_callback and friends (include/chromadec/log.h).
// As in the reference (src/common/log.cpp:30-110): no sink until one is
// installed, threshold INFO, thresholds clamped to [DEBUG, OFF], emits under a
// shared lock so a sink is never replaced while a call into it runs, and the
// sink state is never destroyed so logging stays safe during process exit.
#include <atomic>
#include <iostream>
#include <shared_mutex>
#include <string>

#include "abi_handles.h"
#include "log_sink.h"

namespace chdg {

namespace {

struct SinkState {
    std::shared_mutex mutex;
    chd_log_fn fn = nullptr;
    void *user = nullptr;
};

SinkState &sink()
{
    static SinkState *s = new SinkState();
    return *s;
}

std::atomic<int> g_min_level{CHD_LOG_INFO};
std::atomic<bool> g_have_sink{false};

void stderr_sink(chd_log_level_t level, chd_log_flags_t, const char *message, void *)
{
    std::string line = chd_log_level_str(level);
    line += ": ";
    line += message;
    line += '\n';
    std::cerr << line;
}

bool enabled(int level)
{
    if (level >= CHD_LOG_OFF) return false;
    return g_have_sink.load(std::memory_order_relaxed) && level >= g_min_level.load(std::memory_order_relaxed);
}

}  // namespace

void log_emit(chd_log_level_t level, chd_log_flags_t flags, const char *message)
{
    if (!enabled(level)) return;
    SinkState &s = sink();
    std::shared_lock<std::shared_mutex> l(s.mutex);
    if (s.fn != nullptr) s.fn(level, flags, message, s.user);
}

}  // namespace chdg

CHD_API void chd_set_log_callback(chd_log_fn fn_or_null, void *user_data)
{
    chdg::SinkState &s = chdg::sink();
    std::unique_lock<std::shared_mutex> l(s.mutex);
    s.fn = fn_or_null;
    s.user = user_data;
    chdg::g_have_sink.store(fn_or_null != nullptr, std::memory_order_relaxed);
}

CHD_API void chd_log_to_stderr(void) { chd_set_log_callback(chdg::stderr_sink, nullptr); }

CHD_API void chd_set_log_level(chd_log_level_t min_level)
{
    int l = (int)min_level;
    if (l < CHD_LOG_DEBUG) l = CHD_LOG_DEBUG;
    if (l > CHD_LOG_OFF) l = CHD_LOG_OFF;
    chdg::g_min_level.store(l, std::memory_order_relaxed);
}

CHD_API chd_log_level_t chd_get_log_level(void) { return (chd_log_level_t)chdg::g_min_level.load(); }

CHD_API int chd_log_is_enabled(chd_log_level_t level) { return chdg::enabled(level) ? 1 : 0; }

CHD_API const char *chd_log_level_str(chd_log_level_t level)
{
    switch (level) {
    case CHD_LOG_DEBUG: return "DEBUG";
    case CHD_LOG_INFO: return "INFO";
    case CHD_LOG_WARN: return "WARN";
    case CHD_LOG_ERROR: return "ERROR";
    case CHD_LOG_OFF: return "OFF";
    }
    return "UNKNOWN";
}
