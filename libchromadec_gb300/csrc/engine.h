// engine.h -- the device pipeline behind chromadec_gb300.h and the chd_* ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/chromadec_gb300.h"
#include "masknet.h"
#include "tpal_kernels.h"

namespace chdg {

void output_geometry(const chdg_geometry &g, int padding, int &w, int &h, int &lp, int &tp);

// Frames [a, b) as pipeline batches: one batch when the run fits one,
// otherwise batches of `batch` frames with a first and a last batch of
// `edge` (at most half a batch), so the first upload and the last download
// -- the copies no kernel overlaps -- stay small.
inline std::vector<std::pair<int64_t, int64_t>> edge_batches(int64_t a, int64_t b, int64_t batch, int64_t edge)
{
    std::vector<std::pair<int64_t, int64_t>> out;
    batch = batch > 1 ? batch : 1;
    const int64_t half = batch / 2 > 1 ? batch / 2 : 1;
    edge = edge < half ? (edge > 1 ? edge : 1) : half;
    if (b - a <= batch) {
        if (b > a) out.emplace_back(a, b);
        return out;
    }
    int64_t c = a;
    out.emplace_back(c, c + edge);
    c += edge;
    while (b - c > batch + edge) {
        out.emplace_back(c, c + batch);
        c += batch;
    }
    if (b - c > edge) {
        out.emplace_back(c, b - edge);
        c = b - edge;
    }
    out.emplace_back(c, b);
    return out;
}

class Engine {
public:
    Engine() = default;
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    int init(const chdg_geometry &g, const chdg_config &c);
    // Allocation-free set-up and decode (used by chdg_decode_device_static):
    // the per-bin threshold table and the chroma scratch are caller-provided
    // device memory; nothing is allocated and no counters are kept. A per-bin
    // table is uploaded on `s`, ordered with that stream's earlier decodes.
    int init_static(const chdg_geometry &g, const chdg_config &c, float *thr_table_dev, cudaStream_t s);
    int decode_scratch(const uint16_t *fields, long long stride, int nfields, int fb, int fe, void *out,
                       float *scratch, size_t scratch_floats, cudaStream_t s);
    static size_t scratch_floats_for(const chdg_geometry &g, int nframes);
    // Caller-provided buffers of the guard-band decision passes for the
    // allocation-free decode: records, a list of as many (work item, step)
    // pairs, two counters.
    void set_static_decisions(void *records, unsigned *items, unsigned long long cap, unsigned *counters)
    {
        unc_rec_ = records;
        rerun_ = items;
        unc_cap_ = cap;
        counters_ = counters;
    }
    // Drop the borrowed buffers before destruction (they are not ours to free).
    void forget_static()
    {
        thr_dev_ = nullptr;
        unc_rec_ = nullptr;
        rerun_ = nullptr;
        counters_ = nullptr;
    }
    // fields: device buffer holding capture fields [field_base, ...)
    int decode(const uint16_t *fields, long long stride, int field_base, int nfields, int fb, int fe, void *out,
               cudaStream_t s);
    int chroma(const uint16_t *fields, long long stride, int nfields, int fb, int fe, float *out, cudaStream_t s);
    // Host capture -> host frames: pipelined H2D, decode, D2H.
    int decode_host(const uint16_t *host_fields, long long host_stride, int nfields, int fb, int fe, void *host_out,
                    cudaStream_t s);
    int stats(uint64_t *exact, uint64_t *flips);
    // Per-kernel CUDA-event timing of decode()'s launches.
    void set_profiling(bool on) { profiling_ = on; }
    int kernel_times(double *ms_transform, double *ms_demod, long long *launches);
    void reset_kernel_times();

    int out_w() const { return out_w_; }
    int out_h() const { return out_h_; }
    int left_pad() const { return left_pad_; }
    int top_pad() const { return top_pad_; }
    size_t frame_bytes() const;
    const chdg_geometry &geometry() const { return g_; }
    const chdg_config &config() const { return c_; }
    int look_behind() const { return c_.kind == 8 ? 2 : 0; }   // TransformPal3D::getLookBehind
    int look_ahead() const { return c_.kind == 8 ? 4 : 0; }    // TransformPal3D::getLookAhead
    void set_max_batch_frames(int n) { max_batch_frames_ = n > 0 ? n : 1; }
    void set_chunk_frames(int n) { chunk_frames_ = n > 0 ? n : 1; }
    int chunk_frames() const { return chunk_frames_; }
    // Cap on the 3D transform's grid (0 = one block per 4 work items); a
    // capped grid walks the items persistently.
    void set_max_blocks(int n) { max_blocks3_ = n > 0 ? n : 0; }
    int max_blocks() const { return max_blocks3_; }
    // Tensor-core form of the 3D transform (-1: the plain form, the default;
    // 0: 3xTF32; 1: BF16x3). Transform 3D, uniform threshold only.
    int set_tc_form(int variant);
    int tc_form() const { return tc_variant_; }
    // Learned form (borrowed network; null restores the plain form).
    int set_masknet(MaskNet *net);
    // The learned form's passes with caller buffers (chdg_learned_*).
    int learned_features(const uint16_t *fields, long long stride, int nfields, int fb, int fe, uint16_t *feat,
                         float2 *spec, float *thr_p, cudaStream_t s);
    int learned_chroma(const uint16_t *fields, long long stride, int nfields, int fb, int fe, const float *p,
                       const uint8_t *fallback, float *out, cudaStream_t s);
    int learned_stats(long long *tiles, long long *fallback_tiles);
    // Batches of captures in one frame index space: every field's first
    // sample (null for the black gap fields between captures), every frame's
    // squared threshold (f, hi, lo) and output pointer (null for gap frames).
    // Device arrays indexed by field / frame; null restores the
    // single-capture behaviour.
    void set_frame_tables(const uint16_t *const *d_field_ptrs, const float *d_frame_t2, void *const *d_frame_out)
    {
        field_ptrs_ = d_field_ptrs;
        frame_t2_ = d_frame_t2;
        frame_out_ = d_frame_out;
    }

private:
    bool padded() const { return left_pad_ || top_pad_ || out_w_ != (g_.active_end - g_.active_start) ||
                                 out_h_ != (g_.last_active_frame_line - g_.first_active_frame_line + 1); }
    int ensure_partial(int nout_fields);
    // deferred 3D decisions: record and work-item buffers for a launch of
    // `frames` frames in `nchunks` chunks
    int ensure_deferred(int frames, int nchunks);
    int run_transform(const uint16_t *fields, long long stride, int field_base, int nfields, int fb, int fe,
                      float *partial, cudaStream_t s);
    int run_demod(const uint16_t *fields, long long stride, int field_base, int fb, int fe, const float *partial,
                  void *out, cudaStream_t s);
    // the 3D transform's parameters for frames [fb, fe)
    void t3_params(tpal::T3Params &P, const uint16_t *fields, long long stride, int field_base, int nfields, int fb,
                   int fe, float *partial) const;
    int ensure_host_pipeline(size_t field_bytes, size_t out_bytes);
    void record_pending();
    int fill_border(void *out, int nframes, cudaStream_t s);

    chdg_geometry g_{};
    chdg_config c_{};
    int device_ = 0;
    float t2f_ = 0.f, t2hi_ = 0.f, t2lo_ = 0.f;
    float cfilt_[8][4] = {}, yfilt_[8][2] = {};   // the demodulator's taps for this sample rate
    float *thr_dev_ = nullptr;
    unsigned *stats_dev_ = nullptr;
    float *partial_ = nullptr;
    size_t partial_elems_ = 0;
    bool static_ = false;          // init_static: caller-provided buffers, no allocation
    void *unc_rec_ = nullptr;
    unsigned *rerun_ = nullptr, *counters_ = nullptr;
    unsigned long long unc_cap_ = 0;
    int fl_lo_ = 0, fl_hi_ = 0, rows_ = 0, cols_ = 0;
    int out_w_ = 0, out_h_ = 0, left_pad_ = 0, top_pad_ = 0;
    int max_batch_frames_ = 256;
    int chunk_frames_ = 48;
    int max_blocks3_ = 0;
    int tc_variant_ = -1;
    // learned form: the network (borrowed), per-Z-tile buffers, counters
    MaskNet *net_ = nullptr;
    uint16_t *lfeat_ = nullptr;
    float *lp_ = nullptr;
    uint8_t *lfb_ = nullptr;
    long long lcap_ = 0;
    unsigned long long *lcount_ = nullptr;   // [0] tiles, [1] fallback tiles
    int ensure_learned(long long ntiles);
    int run_learned(const tpal::T3Params &P, cudaStream_t s);
    const uint16_t *const *field_ptrs_ = nullptr;
    const float *frame_t2_ = nullptr;
    void *const *frame_out_ = nullptr;
    // host pipeline: two slots of device fields + frames, one copy stream
    int host_batch_frames_ = 64;
    static constexpr int kHostEdgeFrames = 16;   // the first and last batch of a long run
    uint16_t *hp_fields_[2] = {nullptr, nullptr};
    void *hp_out_[2] = {nullptr, nullptr};
    size_t hp_field_bytes_ = 0, hp_out_bytes_ = 0;
    cudaStream_t copy_stream_ = nullptr, d2h_stream_ = nullptr;
    cudaEvent_t ev_h2d_[2] = {nullptr, nullptr}, ev_comp_[2] = {nullptr, nullptr}, ev_d2h_[2] = {nullptr, nullptr};
    // profiling
    bool profiling_ = false;
    struct Pending { cudaEvent_t a, b, c; };
    std::vector<Pending> pending_;
    double ms_transform_ = 0.0, ms_demod_ = 0.0;
    long long launches_ = 0;
};

}  // namespace chdg
