// masknet.h -- the learned chroma-mask network (masknet.cu) behind
// chdg_masknet_* and the learned form of the Transform-PAL 3D engine.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace chdg {

class MaskNet {
public:
    MaskNet() = default;
    ~MaskNet();
    MaskNet(const MaskNet &) = delete;
    MaskNet &operator=(const MaskNet &) = delete;

    int init();
    int set_weights(const float *host, size_t n);
    int get_weights(float *host, size_t n) const;
    void set_confidence(float limit) { conf_limit_ = limit; }
    // forward passes on the tensor cores (tcgen05, the default) or on the
    // CUDA cores (the SIMT kernel, kept as the cross-check)
    void set_tensor_cores(bool on) { tc_ = on; }
    // wait for `s` and report a tensor-core completion wait that ran out
    int sync(cudaStream_t s) const;
    float confidence() const { return conf_limit_; }
    // p (and fallback flags) of ntiles tiles of features, [tile][1280]
    int forward(const uint16_t *d_feat, long long ntiles, float *d_p, uint8_t *d_fallback, cudaStream_t s) const;
    // Loss and gradients of a batch (ac: per bin |X|^2 and Re(C conj X));
    // lr > 0 then takes one Adam step. loss / host_grad (NPARAM floats), when
    // given, are filled after a stream synchronisation.
    int train_step(const uint16_t *d_feat, const float2 *d_ac, long long ntiles, float lr, double *loss,
                   float *host_grad, cudaStream_t s);

private:
    int ensure_batch(long long ntiles);
    int build_images(cudaStream_t s);
    float *master_ = nullptr, *used_ = nullptr, *m_ = nullptr, *v_ = nullptr, *grad_ = nullptr;
    float *gpart_ = nullptr;
    double *scal_ = nullptr;
    uint16_t *a1_ = nullptr, *a2_ = nullptr, *a3_ = nullptr;
    float *p_ = nullptr, *dz_ = nullptr;
    long long cap_ = 0;
    int grid_ = 1;
    long long step_ = 0;
    float conf_limit_ = 0.1f;
    bool tc_ = true;
    uint8_t *img_ = nullptr;   // bf16 weight images of the tensor-core kernel
    int *err_ = nullptr;
};

}  // namespace chdg

struct chdg_masknet;
namespace chdg {
// The network behind a chdg_masknet handle.
MaskNet *masknet_of(chdg_masknet *n);
}  // namespace chdg
