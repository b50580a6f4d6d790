// abi_errors.cpp -- chd_status_str / chd_last_error / chd_clear_last_error
// (include/chromadec/errors.h; reference: include/chromadec/errors.h:33-41,
// src/abi/c_api_errors.cpp).
#include <chromadec/errors.h>

#include "error_state.h"

#define CHD_API extern "C" __attribute__((visibility("default")))

CHD_API const char *chd_status_str(chd_status_t s)
{
    switch (s) {
    case CHD_OK: return "CHD_OK";
    case CHD_E_INVALID_ARG: return "CHD_E_INVALID_ARG";
    case CHD_E_FILE_NOT_FOUND: return "CHD_E_FILE_NOT_FOUND";
    case CHD_E_IO: return "CHD_E_IO";
    case CHD_E_FORMAT_UNSUPPORTED: return "CHD_E_FORMAT_UNSUPPORTED";
    case CHD_E_METADATA_MISSING: return "CHD_E_METADATA_MISSING";
    case CHD_E_METADATA_CORRUPT: return "CHD_E_METADATA_CORRUPT";
    case CHD_E_PRESET_UNKNOWN: return "CHD_E_PRESET_UNKNOWN";
    case CHD_E_DECODER_UNKNOWN: return "CHD_E_DECODER_UNKNOWN";
    case CHD_E_DECODER_INCOMPATIBLE: return "CHD_E_DECODER_INCOMPATIBLE";
    case CHD_E_NN_MODEL_LOAD: return "CHD_E_NN_MODEL_LOAD";
    case CHD_E_NN_BACKEND_UNAVAILABLE: return "CHD_E_NN_BACKEND_UNAVAILABLE";
    case CHD_E_NN_INFERENCE: return "CHD_E_NN_INFERENCE";
    case CHD_E_OUT_OF_RANGE: return "CHD_E_OUT_OF_RANGE";
    case CHD_E_CANCELLED: return "CHD_E_CANCELLED";
    case CHD_E_INTERNAL: return "CHD_E_INTERNAL";
    case CHD_E_OOM: return "CHD_E_OOM";
    case CHD_E_UNSUPPORTED: return "CHD_E_UNSUPPORTED";
    }
    return "CHD_E_UNKNOWN";
}

CHD_API const char *chd_last_error(void) { return chd::detail::get_last_error().c_str(); }

CHD_API void chd_clear_last_error(void) { chd::detail::clear_last_error(); }
