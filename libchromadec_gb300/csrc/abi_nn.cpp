// abi_nn.cpp -- the NN model calls of the chd_* ABI (include/chromadec/nn.h).
// No NN decoder kinds run here, so these answer as the reference does when
// built without an inference backend (src/abi/c_api_nn.cpp:119-136, 301-339).
#include <chromadec/nn.h>

#include <string>

#include "abi_handles.h"
#include "error_state.h"

namespace {

chd_status_t nn_disabled(const char *what)
{
    chd::detail::set_last_error(std::string("chromadec: ") + what +
                                " requires a build with an NN inference backend; this library has none");
    return CHD_E_INTERNAL;
}

}  // namespace

CHD_API void chd_nn_session_opts_default(chd_nn_session_opts_t *out)
{
    if (out == nullptr) return;
    out->backend = CHD_NN_BACKEND_AUTO;
    out->device_id = 0;
    out->enable_graph_optim = 1;
    out->enable_mem_pattern = 1;
    out->inter_op_threads = 0;
    out->intra_op_threads = 1;
    out->engine_cache_dir = nullptr;
    out->coreml_compute = CHD_NN_COREML_CPU_AND_GPU;
    out->precision = CHD_NN_PRECISION_FP32;
    for (auto &r : out->reserved) r = nullptr;
}

CHD_API chd_status_t chd_nn_model_load_from_file(const char *, const chd_nn_session_opts_t *, chd_nn_model_t **)
{
    return nn_disabled("chd_nn_model_load_from_file");
}

CHD_API chd_status_t chd_nn_model_load_from_memory(const void *, size_t, const chd_nn_session_opts_t *,
                                                   chd_nn_model_t **)
{
    return nn_disabled("chd_nn_model_load_from_memory");
}

CHD_API void chd_nn_model_free(chd_nn_model_t *) {}

CHD_API chd_status_t chd_nn_model_get_active_backend(const chd_nn_model_t *, chd_nn_backend_t *)
{
    return nn_disabled("chd_nn_model_get_active_backend");
}

CHD_API int chd_nn_backend_is_available(chd_nn_backend_t) { return 0; }

CHD_API chd_status_t chd_nn_backend_set_library_path(chd_nn_backend_t backend, const char *)
{
    switch (backend) {
    case CHD_NN_BACKEND_AUTO: case CHD_NN_ORT_AUTO: case CHD_NN_ORT_CPU: case CHD_NN_ORT_CUDA:
    case CHD_NN_ORT_TENSORRT: case CHD_NN_ORT_COREML: case CHD_NN_ORT_DIRECTML: case CHD_NN_ORT_MIGRAPHX:
    case CHD_NN_COREML:
        break;
    default:
        chd::detail::set_last_error("chd_nn_backend_set_library_path: " + std::to_string((int)backend) +
                                    " is not a chd_nn_backend_t value");
        return CHD_E_INVALID_ARG;
    }
    chd::detail::set_last_error("chromadec: chd_nn_backend_set_library_path requires a build with an ONNX Runtime "
                                "backend; this library has none");
    return CHD_E_UNSUPPORTED;
}
