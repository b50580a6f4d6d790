// error_state.h -- the calling thread's last-error detail behind
// chd_last_error() (the reference keeps the same thread-local contract,
// src/common/error_state.cpp).
#pragma once

#include <string>

namespace chd::detail {

void set_last_error(const std::string &msg);
const std::string &get_last_error();
void clear_last_error();

}  // namespace chd::detail
