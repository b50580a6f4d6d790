/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Neural-network model handles (reference: include/chromadec/nn.h). This
 * library has no NN decoder kinds: the calls behave as the reference's build
 * without an inference backend (src/abi/c_api_nn.cpp, the !CHD_WITH_NN
 * branch). The types keep the reference's layout and values so consumers
 * built against its header link unchanged. */
#ifndef CHROMADEC_NN_H
#define CHROMADEC_NN_H

#include <chromadec/enum.h>
#include <chromadec/errors.h>
#include <chromadec/types.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef CHD_ENUM(chd_nn_backend) {
    CHD_NN_BACKEND_AUTO  = 0,
    CHD_NN_ORT_AUTO      = 10,
    CHD_NN_ORT_CPU       = 11,
    CHD_NN_ORT_CUDA      = 12,
    CHD_NN_ORT_TENSORRT  = 13,
    CHD_NN_ORT_COREML    = 14,
    CHD_NN_ORT_DIRECTML  = 15,
    CHD_NN_ORT_MIGRAPHX  = 16,
    CHD_NN_COREML        = 20
} chd_nn_backend_t;

typedef CHD_ENUM(chd_nn_coreml_compute) {
    CHD_NN_COREML_CPU_AND_GPU = 0,
    CHD_NN_COREML_ALL         = 1,
    CHD_NN_COREML_CPU_ONLY    = 2
} chd_nn_coreml_compute_t;

typedef CHD_ENUM(chd_nn_compute_precision) {
    CHD_NN_PRECISION_FP32         = 0,
    CHD_NN_PRECISION_FP16_ALLOWED = 1
} chd_nn_compute_precision_t;

typedef struct chd_nn_session_opts {
    chd_nn_backend_t backend;
    int32_t device_id;
    int     enable_graph_optim;
    int     enable_mem_pattern;
    int32_t inter_op_threads;
    int32_t intra_op_threads;
    chd_nn_coreml_compute_t coreml_compute;
    const char *engine_cache_dir;
    chd_nn_compute_precision_t precision;
    void *reserved[4];
} chd_nn_session_opts_t;

/* Defaults of reference nn.h / c_api_nn.cpp:119-136. */
void chd_nn_session_opts_default(chd_nn_session_opts_t *out);
/* CHD_E_INTERNAL: no inference backend in this build (c_api_nn.cpp:301-324). */
chd_status_t chd_nn_model_load_from_file(const char *model_path, const chd_nn_session_opts_t *opts_or_null,
                                         chd_nn_model_t **out);
chd_status_t chd_nn_model_load_from_memory(const void *model_data, size_t model_size,
                                           const chd_nn_session_opts_t *opts_or_null, chd_nn_model_t **out);
void chd_nn_model_free(chd_nn_model_t *m);
chd_status_t chd_nn_model_get_active_backend(const chd_nn_model_t *m, chd_nn_backend_t *out);
/* 0 for every backend. */
int chd_nn_backend_is_available(chd_nn_backend_t b);
/* CHD_E_INVALID_ARG for a value outside chd_nn_backend_t, else CHD_E_UNSUPPORTED. */
chd_status_t chd_nn_backend_set_library_path(chd_nn_backend_t backend, const char *path_or_null);

#ifdef __cplusplus
}
#endif

#endif
