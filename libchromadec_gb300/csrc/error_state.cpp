// error_state.cpp -- thread-local last-error detail and the status names of
// the chd_* ABI (include/chromadec/errors.h; the reference implements the
// same contract in src/abi/c_api_errors.cpp and src/common/error_state.cpp).
#include "error_state.h"

namespace chd::detail {

static thread_local std::string t_last_error;

void set_last_error(const std::string &msg) { t_last_error = msg; }
const std::string &get_last_error() { return t_last_error; }
void clear_last_error() { t_last_error.clear(); }

}  // namespace chd::detail
