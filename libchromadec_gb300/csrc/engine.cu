// engine.cu -- host side of the device pipeline: geometry, constant tables,
// scratch, launches. Implements include/chromadec_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/chromadec_gb300.h"
#include "engine.h"
#include "error_state.h"
#include "tpal_kernels.h"

namespace tpal {
}

namespace chdg {

static int cuda_fail(const char *what, cudaError_t e)
{
    chd::detail::set_last_error(std::string("chromadec_gb300: ") + what + ": " + cudaGetErrorString(e));
    return CHDG_E_CUDA;
}

// PalColour::MAX_WIDTH (src/decoders/palcolour/palcolour.h:93): the widest
// line the reference decodes
constexpr int kMaxWidth = 1135;

static int arg_fail(const std::string &what)
{
    chd::detail::set_last_error("chromadec_gb300: " + what);
    return CHDG_E_INVALID_ARG;
}


void output_geometry(const chdg_geometry &g, int padding, int &w, int &h, int &lp, int &tp)
{
    // OutputWriter::updateConfiguration, src/output/output_writer.cpp:195-239
    const int aw = g.active_end - g.active_start;
    const int ah = (g.last_active_frame_line - g.first_active_frame_line) + 1;
    int l = 0, r = 0, t = 0, b = 0, ow = aw, oh = ah;
    if (padding > 1) {
        while ((ow % padding) != 0) {
            if ((ow % 2) == 0) r++;
            else l++;
            ow = l + aw + r;
        }
        while ((oh % padding) != 0) {
            if ((oh % 2) == 0) b++;
            else t++;
            oh = t + ah + b;
        }
    }
    w = ow;
    h = oh;
    lp = l;
    tp = t;
}

Engine::~Engine()
{
    if (partial_) cudaFree(partial_);
    if (thr_dev_) cudaFree(thr_dev_);
    if (stats_dev_) cudaFree(stats_dev_);
    if (unc_rec_) cudaFree(unc_rec_);
    if (rerun_) cudaFree(rerun_);
    if (counters_) cudaFree(counters_);
    if (lfeat_) cudaFree(lfeat_);
    if (lp_) cudaFree(lp_);
    if (lfb_) cudaFree(lfb_);
    if (lcount_) cudaFree(lcount_);
    for (int i = 0; i < 2; i++) {
        if (hp_fields_[i]) cudaFree(hp_fields_[i]);
        if (hp_out_[i]) cudaFree(hp_out_[i]);
        if (ev_h2d_[i]) cudaEventDestroy(ev_h2d_[i]);
        if (ev_comp_[i]) cudaEventDestroy(ev_comp_[i]);
        if (ev_d2h_[i]) cudaEventDestroy(ev_d2h_[i]);
    }
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    if (d2h_stream_) cudaStreamDestroy(d2h_stream_);
    reset_kernel_times();
}

int Engine::init(const chdg_geometry &g, const chdg_config &c)
{
    g_ = g;
    c_ = c;
    if (c.kind != 6 && c.kind != 7 && c.kind != 8)
        return arg_fail("kind must be CHD_DEC_PAL_2D (6), CHD_DEC_TRANSFORM_2D (7) or CHD_DEC_TRANSFORM_3D (8)");
    if (g.field_width <= 0 || g.field_height <= 0 || g.active_start < 0 || g.active_end > g.field_width ||
        g.active_end <= g.active_start || g.first_active_frame_line < 0 ||
        g.last_active_frame_line >= 2 * g.field_height - 1 || g.last_active_frame_line < g.first_active_frame_line)
        return arg_fail("invalid geometry");
    if (std::fabs(g.fsc / g.sample_rate - 0.25) > 1e-9)
        return chd::detail::set_last_error("chromadec_gb300: only 4fsc sampling is supported"), CHDG_E_UNSUPPORTED;
    if (g.active_start - 7 < 0 || g.active_end + 8 > kMaxWidth || g.field_width > kMaxWidth)
        return chd::detail::set_last_error("chromadec_gb300: active window too close to the line ends"),
               CHDG_E_UNSUPPORTED;
    if (c.output_format < 0 || c.output_format > 5) return arg_fail("output_format must be 0..5");
    if (c.padding_multiple < 1 || c.padding_multiple > 1024) return arg_fail("padding_multiple out of range");
    if (c.first_field_offset != 0 && c.first_field_offset != 1) return arg_fail("first_field_offset must be 0 or 1");
    if (!(c.y_nr_level >= 0.0)) return arg_fail("y_nr_level must be >= 0");
    const int nthr = (c.kind == 7) ? 80 : 768;
    if (c.kind == 6 && c.thresholds != nullptr) return arg_fail("CHD_DEC_PAL_2D takes no thresholds");
    if (c.thresholds != nullptr && c.n_thresholds != nthr)
        return arg_fail("thresholds table must have " + std::to_string(nthr) + " entries");

    cudaError_t e = cudaGetDevice(&device_);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
    if (c.kind == 8) {
        if (tpal::tp3_init_constants(device_) != 0) return cuda_fail("3D constants", cudaGetLastError());
    } else if (c.kind == 7) {
        if (tpal::tp2_init_constants(device_) != 0) return cuda_fail("2D constants", cudaGetLastError());
    }
    if (tpal::demod_init_constants(device_) != 0) return cuda_fail("demod constants", cudaGetLastError());
    if (tpal::demod_taps(g.sample_rate, cfilt_, yfilt_) != 0)
        return chd::detail::set_last_error("chromadec_gb300: unsupported chroma filter size"), CHDG_E_UNSUPPORTED;

    // Squared thresholds (TransformPal::updateConfiguration, transform_pal.cpp:53-78)
    const double t2 = c.threshold * c.threshold;
    t2f_ = (float)t2;
    t2hi_ = (float)t2;
    t2lo_ = (float)(t2 - (double)t2hi_);
    if (c.thresholds != nullptr) {
        std::vector<float> tab(3 * nthr);
        for (int i = 0; i < nthr; i++) {
            const double v = c.thresholds[i] * c.thresholds[i];
            tab[3 * i] = (float)v;
            tab[3 * i + 1] = (float)v;
            tab[3 * i + 2] = (float)(v - (double)(float)v);
        }
        if ((e = cudaMalloc(&thr_dev_, sizeof(float) * tab.size())) != cudaSuccess) return cuda_fail("cudaMalloc", e);
        if ((e = cudaMemcpy(thr_dev_, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda_fail("cudaMemcpy", e);
    }
    if ((e = cudaMalloc(&stats_dev_, sizeof(unsigned) * 4)) != cudaSuccess) return cuda_fail("cudaMalloc", e);
    cudaMemset(stats_dev_, 0, sizeof(unsigned) * 4);

    fl_lo_ = g.first_active_frame_line / 2;
    fl_hi_ = g.last_active_frame_line / 2 + 1;
    rows_ = fl_hi_ - fl_lo_;
    cols_ = g.active_end - g.active_start;
    output_geometry(g, c.padding_multiple, out_w_, out_h_, left_pad_, top_pad_);
    return 0;
}

int Engine::init_static(const chdg_geometry &g, const chdg_config &c, float *thr_table_dev, cudaStream_t s)
{
    g_ = g;
    c_ = c;
    static_ = true;
    if (c.kind != 8) return arg_fail("the allocation-free decode supports CHD_DEC_TRANSFORM_3D (8) only");
    if (g.field_width <= 0 || g.field_height <= 0 || g.active_start < 0 || g.active_end > g.field_width ||
        g.active_end <= g.active_start || g.first_active_frame_line < 0 ||
        g.last_active_frame_line >= 2 * g.field_height - 1 || g.last_active_frame_line < g.first_active_frame_line)
        return arg_fail("invalid geometry");
    if (std::fabs(g.fsc / g.sample_rate - 0.25) > 1e-9)
        return chd::detail::set_last_error("chromadec_gb300: only 4fsc sampling is supported"), CHDG_E_UNSUPPORTED;
    if (g.active_start - 7 < 0 || g.active_end + 8 > kMaxWidth || g.field_width > kMaxWidth)
        return chd::detail::set_last_error("chromadec_gb300: active window too close to the line ends"),
               CHDG_E_UNSUPPORTED;
    if (c.output_format < 0 || c.output_format > 5) return arg_fail("output_format must be 0..5");
    if (c.padding_multiple < 1 || c.padding_multiple > 1024) return arg_fail("padding_multiple out of range");
    if (c.first_field_offset != 0 && c.first_field_offset != 1) return arg_fail("first_field_offset must be 0 or 1");
    if (!(c.y_nr_level >= 0.0)) return arg_fail("y_nr_level must be >= 0");
    if (c.thresholds != nullptr && c.n_thresholds != 768) return arg_fail("thresholds table must have 768 entries");
    cudaError_t e = cudaGetDevice(&device_);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
    if (tpal::tp3_init_constants(device_) != 0) return cuda_fail("3D constants", cudaGetLastError());
    if (tpal::demod_init_constants(device_) != 0) return cuda_fail("demod constants", cudaGetLastError());
    if (tpal::demod_taps(g.sample_rate, cfilt_, yfilt_) != 0)
        return chd::detail::set_last_error("chromadec_gb300: unsupported chroma filter size"), CHDG_E_UNSUPPORTED;
    const double t2 = c.threshold * c.threshold;
    t2f_ = (float)t2;
    t2hi_ = (float)t2;
    t2lo_ = (float)(t2 - (double)t2hi_);
    thr_dev_ = nullptr;
    if (c.thresholds != nullptr) {
        if (thr_table_dev == nullptr) return arg_fail("no device threshold table");
        float tab[3 * 768];
        for (int i = 0; i < 768; i++) {
            const double v = c.thresholds[i] * c.thresholds[i];
            tab[3 * i] = (float)v;
            tab[3 * i + 1] = (float)v;
            tab[3 * i + 2] = (float)(v - (double)(float)v);
        }
        // On the caller's stream: a decode still queued there reads the table
        // of its own call before this copy replaces it. The source is
        // pageable, so the call returns once it has been staged and the stack
        // array may go.
        if ((e = cudaMemcpyAsync(thr_table_dev, tab, sizeof(tab), cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
        thr_dev_ = thr_table_dev;
    }
    stats_dev_ = nullptr;
    fl_lo_ = g.first_active_frame_line / 2;
    fl_hi_ = g.last_active_frame_line / 2 + 1;
    rows_ = fl_hi_ - fl_lo_;
    cols_ = g.active_end - g.active_start;
    output_geometry(g, c.padding_multiple, out_w_, out_h_, left_pad_, top_pad_);
    return 0;
}

size_t Engine::scratch_floats_for(const chdg_geometry &g, int nframes)
{
    const size_t rows = (size_t)(g.last_active_frame_line / 2 + 1 - g.first_active_frame_line / 2);
    const size_t cols = (size_t)(g.active_end - g.active_start);
    return (size_t)4 * 2 * (size_t)nframes * rows * cols;
}

int Engine::decode_scratch(const uint16_t *fields, long long stride, int nfields, int fb, int fe, void *out,
                           float *scratch, size_t scratch_floats, cudaStream_t s)
{
    if (fields == nullptr || out == nullptr || scratch == nullptr || fe < fb ||
        stride < (long long)g_.field_width * g_.field_height)
        return arg_fail("decode: bad arguments");
    if (fe == fb) return 0;
    if (scratch_floats_for(g_, fe - fb) > scratch_floats)
        return arg_fail("decode: " + std::to_string(fe - fb) + " frames exceed the static chroma scratch");
    if (const int rc = run_transform(fields, stride, 0, nfields, fb, fe, scratch, s); rc != 0) return rc;
    return run_demod(fields, stride, 0, fb, fe, scratch, out, s);
}

// Elements per output frame and their size: three planes (or interleaved
// R'G'B') except the gray formats; float for yuv444ps, rgbs and grays.
static size_t format_planes(int fmt) { return (fmt == 4 || fmt == 5) ? 1 : 3; }
static size_t format_elem(int fmt) { return (fmt == 1 || fmt == 3 || fmt == 5) ? sizeof(float) : sizeof(uint16_t); }

size_t Engine::frame_bytes() const
{
    return (size_t)out_w_ * out_h_ * format_planes(c_.output_format) * format_elem(c_.output_format);
}

int Engine::ensure_partial(int nout_fields)
{
    const size_t need = (size_t)4 * nout_fields * rows_ * cols_;
    if (need <= partial_elems_) return 0;
    if (partial_) cudaFree(partial_);
    partial_ = nullptr;
    partial_elems_ = 0;
    cudaError_t e = cudaMalloc(&partial_, need * sizeof(float));
    if (e != cudaSuccess) {
        chd::detail::set_last_error("chromadec_gb300: out of device memory for chroma scratch");
        return CHDG_E_OOM;
    }
    partial_elems_ = need;
    return 0;
}

int Engine::ensure_deferred(int frames, int nchunks)
{
    const int ntiles = ((g_.active_end - (g_.active_start - 8) + 7) / 8) *
                       ((g_.last_active_frame_line - (g_.first_active_frame_line - 16)) / 16 + 1);
    const unsigned long long need = tpal::tp3_unc_capacity(ntiles, frames, nchunks);
    cudaError_t e;
    if (counters_ == nullptr && (e = cudaMalloc(&counters_, 2 * sizeof(unsigned))) != cudaSuccess) {
        counters_ = nullptr;
        return cuda_fail("decision counters", e);
    }
    if (need <= unc_cap_) return 0;
    if (unc_rec_) cudaFree(unc_rec_);
    if (rerun_) cudaFree(rerun_);
    unc_rec_ = nullptr;
    rerun_ = nullptr;
    unc_cap_ = 0;
    // every kx group of every step can hold a record, and each record lists
    // at most one work item
    if ((e = cudaMalloc(&unc_rec_, need * sizeof(tpal::UncRecord))) != cudaSuccess ||
        (e = cudaMalloc(&rerun_, 2 * need * sizeof(unsigned))) != cudaSuccess) {
        if (unc_rec_) cudaFree(unc_rec_);
        unc_rec_ = nullptr;
        rerun_ = nullptr;
        return cuda_fail("decision records", e);
    }
    unc_cap_ = need;
    return 0;
}

void Engine::t3_params(tpal::T3Params &P, const uint16_t *fields, long long stride, int field_base, int nfields,
                       int fb, int fe, float *partial) const
{
    const long long cls_stride = (long long)(fe - fb) * 2 * rows_ * cols_;
    P.fields = fields;
    P.field_ptrs = field_ptrs_;
    P.field_stride = stride;
    P.field_base = field_base;
    P.nfields = nfields;
    P.fw = g_.field_width;
    P.fh = g_.field_height;
    P.avs = g_.active_start;
    P.ave = g_.active_end;
    P.fafl = g_.first_active_frame_line;
    P.lafl = g_.last_active_frame_line;
    P.black = g_.black;
    P.swap = c_.first_field_offset;
    // transform_pal_3d.cpp:151-153 tile grid
    P.tileX0 = g_.active_start - 8;
    P.ntx = (g_.active_end - P.tileX0 + 7) / 8;
    P.tileY0 = g_.first_active_frame_line - 16;
    P.nty = (g_.last_active_frame_line - P.tileY0) / 16 + 1;
    P.frame_begin = fb;
    P.frame_end = fe;
    P.chunk_frames = chunk_frames_;
    P.nchunks = (fe - fb + chunk_frames_ - 1) / chunk_frames_;
    P.partial = partial;
    P.part_class_stride = cls_stride;
    P.part_field_stride = (long long)rows_ * cols_;
    P.part_row_stride = cols_;
    P.fl_lo = fl_lo_;
    P.t2f = t2f_;
    P.t2hi = t2hi_;
    P.t2lo = t2lo_;
    P.thr_table = thr_dev_;
    P.frame_t2 = frame_t2_;
    P.stats = stats_dev_;
}

int Engine::run_transform(const uint16_t *fields, long long stride, int field_base, int nfields, int fb, int fe,
                          float *partial, cudaStream_t s)
{
    const long long cls_stride = (long long)(fe - fb) * 2 * rows_ * cols_;
    if (c_.kind == 6) return 0;   // the PALcolour filter demodulates the composite directly
    if (c_.kind == 8) {
        tpal::T3Params P{};
        t3_params(P, fields, stride, field_base, nfields, fb, fe, partial);
        if (tc_variant_ >= 0) return tpal::tc3_transform(P, g_.field_height, tc_variant_, s);
        if (net_ != nullptr) return run_learned(P, s);
        // guard-band decisions: recorded by the walk, decided by the resolve
        // pass, work items with a wrong FP32 decision walked again exactly
        if (static_) {
            const int ntiles = P.ntx * P.nty;
            if (unc_rec_ == nullptr || tpal::tp3_unc_capacity(ntiles, fe - fb, P.nchunks) > unc_cap_)
                return arg_fail("decode: the static decision records are too small for this picture");
        } else if (const int rc = ensure_deferred(fe - fb, P.nchunks); rc != 0) {
            return rc;
        }
        P.unc_rec = static_cast<tpal::UncRecord *>(unc_rec_);
        P.rerun = rerun_;
        P.counters = counters_;
        P.unc_cap = (unsigned)std::min<unsigned long long>(unc_cap_, 0xFFFFFFFFull);
        if (cudaError_t e = cudaMemsetAsync(counters_, 0, 2 * sizeof(unsigned), s); e != cudaSuccess)
            return cuda_fail("decision counters", e);
        if (tpal::tp3_launch(P, s, max_blocks3_) != 0) return cuda_fail("tpal3d launch", cudaGetLastError());
        if (tpal::tp3_resolve_launch(P, s) != 0) return cuda_fail("tpal3d resolve", cudaGetLastError());
    } else {
        tpal::T2Params P{};
        P.fields = fields;
        P.field_ptrs = field_ptrs_;
        P.field_stride = stride;
        P.field_base = field_base;
        P.nfields = nfields;
        P.fw = g_.field_width;
        P.avs = g_.active_start;
        P.ave = g_.active_end;
        P.fafl = g_.first_active_frame_line;
        P.lafl = g_.last_active_frame_line;
        P.black = g_.black;
        P.swap = c_.first_field_offset;
        P.field_begin = 2 * fb;
        P.nout = 2 * (fe - fb);
        P.partial = partial;
        P.part_class_stride = cls_stride;
        P.part_field_stride = (long long)rows_ * cols_;
        P.part_row_stride = cols_;
        P.fl_lo = fl_lo_;
        P.t2f = t2f_;
        P.t2hi = t2hi_;
        P.t2lo = t2lo_;
        P.thr_table = thr_dev_;
        P.frame_t2 = frame_t2_;
        P.stats = stats_dev_;
        if (tpal::tp2_launch(P, s) != 0) return cuda_fail("tpal2d launch", cudaGetLastError());
    }
    return 0;
}

int Engine::run_demod(const uint16_t *fields, long long stride, int field_base, int fb, int fe, const float *partial,
                      void *out, cudaStream_t s)
{
    tpal::DemodParams D{};
    D.fields = fields;
    D.field_ptrs = field_ptrs_;
    D.field_stride = stride;
    D.field_base = field_base;
    D.field_begin = 2 * fb;
    D.nout = 2 * (fe - fb);
    D.fw = g_.field_width;
    D.fh = g_.field_height;
    D.avs = g_.active_start;
    D.ave = g_.active_end;
    D.fafl = g_.first_active_frame_line;
    D.lafl = g_.last_active_frame_line;
    D.burst_start = g_.burst_start;
    D.burst_end = g_.burst_end;
    D.black = g_.black;
    D.white = g_.white;
    D.partial = (c_.kind == 6) ? nullptr : partial;
    D.part_class_stride = (long long)(fe - fb) * 2 * rows_ * cols_;
    D.part_field_stride = (long long)rows_ * cols_;
    D.part_row_stride = cols_;
    D.fl_lo = fl_lo_;
    D.nclasses = 4;
    D.swap = c_.first_field_offset;
    const double th = (c_.chroma_phase_deg * M_PI) / 180;
    D.gain_cos = (float)(cos(th) * c_.chroma_gain);
    D.gain_sin = (float)(sin(th) * c_.chroma_gain);
    // doYNR coring level: yNRLevel * ((white - black) / 100), the division in
    // integers as in the reference (palcolour.cpp:415-416)
    D.nr_y = (float)(c_.y_nr_level * (double)((g_.white - g_.black) / 100));
    const int fmt = c_.output_format;
    D.format = fmt;
    D.out = out;
    D.frame_out = frame_out_;
    D.out_frame_stride = (long long)out_w_ * out_h_ * (long long)format_planes(fmt);
    D.out_w = out_w_;
    D.out_h = out_h_;
    D.left_pad = left_pad_;
    D.top_pad = top_pad_;
    const double range = (double)(g_.white - g_.black);
    D.ey_scale = (float)(1.0 / range);
    D.ecb_scale = (float)(c_.ecb_from_u / range);
    D.ecr_scale = (float)(c_.ecr_from_v / range);
    auto split = [](double v, float &hi, float &lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    };
    split(219.0 * 256.0 / range, D.qy_hi, D.qy_lo);
    split(224.0 * 256.0 * c_.ecb_from_u / range, D.qcb_hi, D.qcb_lo);
    split(224.0 * 256.0 * c_.ecr_from_v / range, D.qcr_hi, D.qcr_lo);
    // output_writer.cpp:84-143 Y'CbCr clamp bounds
    if (fmt == 1 || fmt == 5) {
        switch (c_.clamp_mode) {
        case 1: D.y_lo = 0.f; D.y_hi = 1.f; D.c_lo = -0.5f; D.c_hi = 0.5f; break;
        case 3: D.y_lo = -15.0f / 219.0f; D.y_hi = 238.75f / 219.0f; D.c_lo = -127.0f / 224.0f; D.c_hi = 126.75f / 224.0f; break;
        default: D.y_lo = -INFINITY; D.y_hi = INFINITY; D.c_lo = -INFINITY; D.c_hi = INFINITY;
        }
    } else {
        switch (c_.clamp_mode) {
        case 1: D.y_lo = 16.f * 256.f; D.y_hi = 235.f * 256.f; D.c_lo = 16.f * 256.f; D.c_hi = 240.f * 256.f; break;
        case 3: D.y_lo = 256.f; D.y_hi = 254.75f * 256.f; D.c_lo = 256.f; D.c_hi = 254.75f * 256.f; break;
        default: D.y_lo = 0.f; D.y_hi = 65535.f; D.c_lo = 0.f; D.c_hi = 65535.f;
        }
    }
    // R'G'B': ColorConversion's matrix (color_conversion.cpp:60-64) and the
    // floatRGBBounds box (output_writer.cpp:149-190)
    const double kg = 1.0 - c_.kr - c_.kb;
    D.r_from_v = (float)(1.0 / c_.v_reduction);
    D.g_from_u = (float)(-(c_.kb / kg) / c_.u_reduction);
    D.g_from_v = (float)(-(c_.kr / kg) / c_.v_reduction);
    D.b_from_u = (float)(1.0 / c_.u_reduction);
    D.rgb_y_scale = (float)(65535.0 / range);
    D.rgb_uv_scale = (float)((fmt == 2 ? 65535.0 : 1.0) / range);
    {
        const float inf = INFINITY;
        float b[6] = {-inf, inf, -inf, inf, -inf, inf};
        if (c_.clamp_mode == 1) {
            for (int i = 0; i < 3; i++) b[2 * i] = 0.f, b[2 * i + 1] = 1.f;
        } else if (c_.clamp_mode == 2) {
            for (int i = 0; i < 3; i++) b[2 * i] = 0.f, b[2 * i + 1] = inf;
        } else if (c_.clamp_mode == 3) {
            const float eyLo = -15.0f / 219.0f, eyHi = 238.75f / 219.0f;
            const float ecLo = -127.0f / 224.0f, ecHi = 126.75f / 224.0f;
            const double bds = 2.0 * (1.0 - c_.kb), rds = 2.0 * (1.0 - c_.kr);
            const double gcb = (c_.kb * bds) / kg, gcr = (c_.kr * rds) / kg;
            b[0] = (float)(eyLo + rds * ecLo);
            b[1] = (float)(eyHi + rds * ecHi);
            b[2] = (float)(eyLo - (gcb + gcr) * ecHi);
            b[3] = (float)(eyHi - (gcb + gcr) * ecLo);
            b[4] = (float)(eyLo + bds * ecLo);
            b[5] = (float)(eyHi + bds * ecHi);
        }
        D.r_lo = b[0], D.r_hi = b[1], D.g_lo = b[2], D.g_hi = b[3], D.b_lo = b[4], D.b_hi = b[5];
    }
    std::memcpy(D.cfilt, cfilt_, sizeof(cfilt_));
    std::memcpy(D.yfilt, yfilt_, sizeof(yfilt_));
    D.swap_carrier = g_.field_height == 263 ? 1 : 0;   // palcolour.cpp:158-173 keys on fieldHeight
    if (padded() && frame_out_ == nullptr) {
        // black border: Y 16*256 / Cb,Cr 128*256 (p16), zeros (ps)
        const int rc = fill_border(out, fe - fb, s);
        if (rc != 0) return rc;
    }
    const int rc = tpal::demod_launch(D, s);
    if (rc != 0) return cuda_fail("demod launch", cudaGetLastError());
    return 0;
}

// Black border of padded frames (OutputWriter::fillBlack, output_writer.cpp:371-400):
// Y 16*256 and Cb/Cr 128*256 for yuv444p16, 16*256 for gray16, zero for
// rgb48 and every float format.
__global__ void fill_frames_kernel(uint16_t *o16, float *o32, long long frame_elems, long long plane, long long nframes,
                                   uint16_t y, uint16_t c)
{
    const long long n = nframes * frame_elems;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (o16) o16[i] = (((i % frame_elems) / plane) == 0) ? y : c;
        else o32[i] = 0.f;
    }
}

int Engine::fill_border(void *out, int nframes, cudaStream_t s)
{
    const int fmt = c_.output_format;
    const long long plane = (long long)out_w_ * out_h_;
    const long long elems = plane * (long long)format_planes(fmt);
    if (format_elem(fmt) == sizeof(float))
        fill_frames_kernel<<<1024, 256, 0, s>>>(nullptr, (float *)out, elems, plane, nframes, 0, 0);
    else if (fmt == 2)
        fill_frames_kernel<<<1024, 256, 0, s>>>((uint16_t *)out, nullptr, elems, plane, nframes, 0, 0);
    else
        fill_frames_kernel<<<1024, 256, 0, s>>>((uint16_t *)out, nullptr, elems, plane, nframes, 16 * 256, 128 * 256);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cuda_fail("fill", e);
}

int Engine::set_masknet(MaskNet *net)
{
    if (net != nullptr && (c_.kind != 8 || thr_dev_ != nullptr || static_ || tc_variant_ >= 0))
        return arg_fail("set_masknet: the learned form is Transform 3D, plain FP32 form, uniform threshold");
    net_ = net;
    return 0;
}

int Engine::ensure_learned(long long ntiles)
{
    cudaError_t e;
    if (lcount_ == nullptr) {
        if ((e = cudaMalloc(&lcount_, 2 * sizeof(unsigned long long))) != cudaSuccess) {
            lcount_ = nullptr;
            return cuda_fail("learned counters", e);
        }
        cudaMemset(lcount_, 0, 2 * sizeof(unsigned long long));
    }
    if (ntiles <= lcap_) return 0;
    if (lfeat_) cudaFree(lfeat_);
    if (lp_) cudaFree(lp_);
    if (lfb_) cudaFree(lfb_);
    lfeat_ = nullptr;
    lp_ = nullptr;
    lfb_ = nullptr;
    lcap_ = 0;
    if ((e = cudaMalloc(&lfeat_, sizeof(uint16_t) * CHDG_MASKNET_BINS * (size_t)ntiles)) != cudaSuccess ||
        (e = cudaMalloc(&lp_, sizeof(float) * CHDG_MASKNET_BINS * (size_t)ntiles)) != cudaSuccess ||
        (e = cudaMalloc(&lfb_, (size_t)ntiles)) != cudaSuccess) {
        chd::detail::set_last_error("chromadec_gb300: out of device memory for the learned form's tile buffers");
        return CHDG_E_OOM;
    }
    lcap_ = ntiles;
    return 0;
}

__global__ void sum_classes_kernel(const float *part, long long cls_stride, long long n, float *out);

__global__ void count_fallback_kernel(const uint8_t *fb, long long n, unsigned long long *count)
{
    unsigned long long c = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c += fb[i];
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) c += __shfl_xor_sync(0xffffffffu, c, h);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count + 1, c);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(count, (unsigned long long)n);
}

// Feature pass, network, apply pass over the Z tiles of frames [fb, fe).
int Engine::run_learned(const tpal::T3Params &P, cudaStream_t s)
{
    const long long ntiles = (long long)P.ntx * P.nty * (long long)(P.frame_end - P.frame_begin + 2);
    if (const int rc = ensure_learned(ntiles); rc != 0) return rc;
    tpal::T3Learn L{};
    L.feat = lfeat_;
    L.z0 = P.frame_begin - 2;
    if (tpal::tp3_learned_launch(P, L, 0, s) != 0) return cuda_fail("learned features", cudaGetLastError());
    if (const int rc = net_->forward(lfeat_, ntiles, lp_, lfb_, s); rc != 0) return rc;
    count_fallback_kernel<<<64, 256, 0, s>>>(lfb_, ntiles, lcount_);
    L.p = lp_;
    L.fallback = lfb_;
    if (tpal::tp3_learned_launch(P, L, 1, s) != 0) return cuda_fail("learned apply", cudaGetLastError());
    return 0;
}

int Engine::learned_features(const uint16_t *fields, long long stride, int nfields, int fb, int fe, uint16_t *feat,
                             float2 *spec, float *thr_p, cudaStream_t s)
{
    if (c_.kind != 8) return arg_fail("learned_features: Transform 3D only");
    if (fields == nullptr || feat == nullptr || fe < fb || stride < (long long)g_.field_width * g_.field_height)
        return arg_fail("learned_features: bad arguments");
    if (fe == fb) return 0;
    tpal::T3Params P{};
    t3_params(P, fields, stride, 0, nfields, fb, fe, nullptr);
    tpal::T3Learn L{};
    L.feat = feat;
    L.spec = spec;
    L.plain_p = thr_p;
    L.z0 = fb - 2;
    return tpal::tp3_learned_launch(P, L, 0, s) == 0 ? 0 : cuda_fail("learned features", cudaGetLastError());
}

int Engine::learned_chroma(const uint16_t *fields, long long stride, int nfields, int fb, int fe, const float *p,
                           const uint8_t *fallback, float *out, cudaStream_t s)
{
    if (c_.kind != 8) return arg_fail("learned_chroma: Transform 3D only");
    if (fields == nullptr || p == nullptr || fallback == nullptr || out == nullptr || fe < fb)
        return arg_fail("learned_chroma: bad arguments");
    if (fe == fb) return 0;
    if (const int rc = ensure_partial(2 * (fe - fb)); rc != 0) return rc;
    tpal::T3Params P{};
    t3_params(P, fields, stride, 0, nfields, fb, fe, partial_);
    tpal::T3Learn L{};
    L.p = p;
    L.fallback = fallback;
    L.z0 = fb - 2;
    if (tpal::tp3_learned_launch(P, L, 1, s) != 0) return cuda_fail("learned apply", cudaGetLastError());
    const long long n = (long long)(fe - fb) * 2 * rows_ * cols_;
    sum_classes_kernel<<<1024, 256, 0, s>>>(partial_, n, n, out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cuda_fail("sum", e);
}

int Engine::learned_stats(long long *tiles, long long *fallback_tiles)
{
    unsigned long long h[2] = {0, 0};
    if (lcount_ != nullptr) {
        cudaError_t e = cudaMemcpy(h, lcount_, sizeof(h), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail("learned stats", e);
    }
    if (tiles) *tiles = (long long)h[0];
    if (fallback_tiles) *fallback_tiles = (long long)h[1];
    return 0;
}

int Engine::set_tc_form(int variant)
{
    if (variant < -1 || variant > 1) return arg_fail("set_tc_form: variant must be -1, 0 or 1");
    if (variant >= 0 && (c_.kind != 8 || thr_dev_ != nullptr || static_ || net_ != nullptr))
        return arg_fail("set_tc_form: the tensor-core form is Transform 3D with a uniform threshold");
    tc_variant_ = variant;
    return 0;
}

int Engine::decode(const uint16_t *fields, long long stride, int field_base, int nfields, int fb, int fe, void *out,
                   cudaStream_t s)
{
    if (fields == nullptr || out == nullptr || fe < fb || stride < (long long)g_.field_width * g_.field_height)
        return arg_fail("decode: bad arguments");
    const int maxb = max_batch_frames_;
    char *o = (char *)out;
    for (int b = fb; b < fe; b += maxb) {
        const int be = std::min(fe, b + maxb);
        if (c_.kind != 6)
            if (const int rc = ensure_partial(2 * (be - b)); rc != 0) return rc;
        Pending ev{};
        if (profiling_) {
            cudaEventCreate(&ev.a);
            cudaEventCreate(&ev.b);
            cudaEventCreate(&ev.c);
            cudaEventRecord(ev.a, s);
        }
        if (const int rc = run_transform(fields, stride, field_base, nfields, b, be, partial_, s); rc != 0) return rc;
        if (profiling_) cudaEventRecord(ev.b, s);
        if (const int rc = run_demod(fields, stride, field_base, b, be, partial_, o, s); rc != 0) return rc;
        if (profiling_) {
            cudaEventRecord(ev.c, s);
            pending_.push_back(ev);
        }
        // transform (+ resolve and apply when deferred) and demodulator;
        // PALcolour runs the demodulator alone
        launches_ += (c_.kind == 6) ? 1
                     : (c_.kind == 8) ? (tc_variant_ >= 0 ? tpal::tc3_launches_per_frames(be - b) + 1 : net_ ? 5 : 4)
                                      : 2;
        o += frame_bytes() * (size_t)(be - b);
    }
    return 0;
}

void Engine::record_pending()
{
    for (auto &p : pending_) {
        float t1 = 0.f, t2 = 0.f;
        cudaEventSynchronize(p.c);
        cudaEventElapsedTime(&t1, p.a, p.b);
        cudaEventElapsedTime(&t2, p.b, p.c);
        ms_transform_ += t1;
        ms_demod_ += t2;
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
        cudaEventDestroy(p.c);
    }
    pending_.clear();
}

int Engine::kernel_times(double *ms_transform, double *ms_demod, long long *launches)
{
    record_pending();
    if (ms_transform) *ms_transform = ms_transform_;
    if (ms_demod) *ms_demod = ms_demod_;
    if (launches) *launches = launches_;
    return 0;
}

void Engine::reset_kernel_times()
{
    record_pending();
    ms_transform_ = ms_demod_ = 0.0;
    launches_ = 0;
}

int Engine::ensure_host_pipeline(size_t field_bytes, size_t out_bytes)
{
    cudaError_t e;
    if (copy_stream_ == nullptr) {
        if ((e = cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail("stream", e);
        if ((e = cudaStreamCreateWithFlags(&d2h_stream_, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail("stream", e);
        for (int i = 0; i < 2; i++) {
            cudaEventCreateWithFlags(&ev_h2d_[i], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&ev_comp_[i], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&ev_d2h_[i], cudaEventDisableTiming);
        }
    }
    if (field_bytes > hp_field_bytes_) {
        for (int i = 0; i < 2; i++) {
            if (hp_fields_[i]) cudaFree(hp_fields_[i]);
            hp_fields_[i] = nullptr;
            if ((e = cudaMalloc(&hp_fields_[i], field_bytes)) != cudaSuccess) {
                hp_field_bytes_ = 0;
                chd::detail::set_last_error("chromadec_gb300: out of device memory for the field ring");
                return CHDG_E_OOM;
            }
        }
        hp_field_bytes_ = field_bytes;
    }
    if (out_bytes > hp_out_bytes_) {
        for (int i = 0; i < 2; i++) {
            if (hp_out_[i]) cudaFree(hp_out_[i]);
            hp_out_[i] = nullptr;
            if ((e = cudaMalloc(&hp_out_[i], out_bytes)) != cudaSuccess) {
                hp_out_bytes_ = 0;
                chd::detail::set_last_error("chromadec_gb300: out of device memory for output frames");
                return CHDG_E_OOM;
            }
        }
        hp_out_bytes_ = out_bytes;
    }
    return 0;
}

// Batches alternate between two device slots: the copy stream uploads batch
// i+1's field window while the compute stream decodes batch i, and downloads
// batch i-1's frames. Batches of B frames, with a first and a last batch of
// at most kHostEdgeFrames (the first upload and the last download are the
// copies no kernel overlaps). A batch's window is its fields plus the 3D
// look-behind/ahead halo (frames b-2 .. b+B+3), clipped to the capture.
int Engine::decode_host(const uint16_t *host_fields, long long host_stride, int nfields, int fb, int fe,
                        void *host_out, cudaStream_t s)
{
    if (host_fields == nullptr || host_out == nullptr || fe < fb) return arg_fail("decode_host: bad arguments");
    const long long flen = (long long)g_.field_width * g_.field_height;
    if (host_stride < flen) return arg_fail("decode_host: field stride smaller than a field");
    const int B = host_batch_frames_;
    const long long dstride = (flen + 63) & ~63LL;   // 128-byte aligned device fields
    const int maxWinFields = 2 * (B + look_behind() + look_ahead());
    if (const int rc = ensure_host_pipeline((size_t)(maxWinFields + 1) * dstride * 2, frame_bytes() * (size_t)B);
        rc != 0)
        return rc;
    cudaError_t e;
    const std::vector<std::pair<int64_t, int64_t>> batches = edge_batches(fb, fe, B, kHostEdgeFrames);
    for (int i = 0; i < (int)batches.size(); i++) {
        const int b = (int)batches[i].first, be = (int)batches[i].second;
        const int slot = i & 1;
        const int f0 = std::max(0, 2 * (b - look_behind()));
        const int f1 = std::min(nfields, 2 * (be + look_ahead()));
        // slot reuse: the slot's previous decode -- batch i-2's, or for the
        // first two batches the previous call's, which may still be running
        // -- must be done before its fields are overwritten (an event never
        // recorded makes the wait a no-op)
        cudaStreamWaitEvent(copy_stream_, ev_comp_[slot], 0);
        if (f1 > f0) {
            e = cudaMemcpy2DAsync(hp_fields_[slot], dstride * 2, host_fields + (size_t)f0 * host_stride,
                                  host_stride * 2, flen * 2, f1 - f0, cudaMemcpyHostToDevice, copy_stream_);
            if (e != cudaSuccess) return cuda_fail("H2D", e);
        }
        cudaEventRecord(ev_h2d_[slot], copy_stream_);
        cudaStreamWaitEvent(s, ev_h2d_[slot], 0);
        cudaStreamWaitEvent(s, ev_d2h_[slot], 0);   // output slot drained (this call's or the previous one's)
        if (const int rc = decode(hp_fields_[slot], dstride, f0, nfields, b, be, hp_out_[slot], s); rc != 0) return rc;
        cudaEventRecord(ev_comp_[slot], s);
        // downloads on their own stream, so the next upload does not queue behind them
        cudaStreamWaitEvent(d2h_stream_, ev_comp_[slot], 0);
        e = cudaMemcpyAsync((char *)host_out + frame_bytes() * (size_t)(b - fb), hp_out_[slot],
                            frame_bytes() * (size_t)(be - b), cudaMemcpyDeviceToHost, d2h_stream_);
        if (e != cudaSuccess) return cuda_fail("D2H", e);
        cudaEventRecord(ev_d2h_[slot], d2h_stream_);
    }
    // the caller's stream completes after the last download
    cudaEventRecord(ev_d2h_[0], d2h_stream_);
    cudaStreamWaitEvent(s, ev_d2h_[0], 0);
    return 0;
}

__global__ void sum_classes_kernel(const float *part, long long cls_stride, long long n, float *out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = part[i] + part[i + cls_stride] + part[i + 2 * cls_stride] + part[i + 3 * cls_stride];
}

int Engine::chroma(const uint16_t *fields, long long stride, int nfields, int fb, int fe, float *out, cudaStream_t s)
{
    if (fields == nullptr || out == nullptr || fe < fb) return arg_fail("chroma: bad arguments");
    if (c_.kind == 6) return arg_fail("chroma: CHD_DEC_PAL_2D has no Transform-PAL stage");
    if (const int rc = ensure_partial(2 * (fe - fb)); rc != 0) return rc;
    if (const int rc = run_transform(fields, stride, 0, nfields, fb, fe, partial_, s); rc != 0) return rc;
    const long long n = (long long)(fe - fb) * 2 * rows_ * cols_;
    sum_classes_kernel<<<1024, 256, 0, s>>>(partial_, n, n, out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cuda_fail("sum", e);
}

int Engine::stats(uint64_t *exact, uint64_t *flips)
{
    unsigned h[4];
    cudaError_t e = cudaMemcpy(h, stats_dev_, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("stats", e);
    if (exact) *exact = h[0];
    if (flips) *flips = h[1];
    return 0;
}

}  // namespace chdg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct chdg_engine {
    chdg::Engine eng;
};

#pragma GCC visibility push(default)
extern "C" {

void chdg_default_geometry(chdg_geometry *g)
{
    if (!g) return;
    // src/format/video_standards.cpp:58-70,116-207 (line-locked PAL preset);
    // active frame lines from src/metadata/core.cpp:40-50.
    g->field_width = 1135;
    g->field_height = 313;
    g->active_start = 177;
    g->active_end = 1125;
    g->first_active_frame_line = 44;
    g->last_active_frame_line = 619;
    g->burst_start = 98;
    g->burst_end = 138;
    g->black = 256 * 64;
    g->white = 844 * 64;
    g->sample_rate = 4.0 * 625.0 * 25.0 * (1135.0 / 4.0 + 1.0 / 625.0);
    g->fsc = 283.75 * 15625.0 + 25.0;
}

void chdg_default_config(chdg_config *c, int32_t kind)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->kind = kind;
    c->threshold = 0.4;
    c->chroma_gain = 1.0;
    c->chroma_phase_deg = 0.0;
    c->output_format = 0;
    c->clamp_mode = 0;
    c->padding_multiple = 1;
    // src/common/color_conversion.cpp:33-66 at Modern / Scientific
    c->kb = 0.114;
    c->kr = 0.299;
    c->u_reduction = 0.49211104112248356308804691718185;
    c->v_reduction = 0.87728321993817866838972487283129;
    c->ecb_from_u = 1.0 / ((2.0 * (1.0 - c->kb)) * c->u_reduction);
    c->ecr_from_v = 1.0 / ((2.0 * (1.0 - c->kr)) * c->v_reduction);
    c->y_nr_level = 0.0;
    c->first_field_offset = 0;
}

int chdg_engine_create(const chdg_geometry *g, const chdg_config *c, chdg_engine **out)
{
    if (!g || !c || !out) return chdg::arg_fail("chdg_engine_create: null argument");
    *out = nullptr;
    auto e = std::make_unique<chdg_engine>();
    if (const int rc = e->eng.init(*g, *c); rc != 0) return rc;
    *out = e.release();
    return 0;
}

void chdg_engine_free(chdg_engine *e) { delete e; }

int chdg_output_geometry(const chdg_engine *e, int32_t *width, int32_t *height, size_t *frame_bytes)
{
    if (!e) return chdg::arg_fail("chdg_output_geometry: null engine");
    if (width) *width = e->eng.out_w();
    if (height) *height = e->eng.out_h();
    if (frame_bytes) *frame_bytes = e->eng.frame_bytes();
    return 0;
}

int chdg_decode_device(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                       int32_t frame_begin, int32_t frame_end, void *d_out, void *stream)
{
    if (!e) return chdg::arg_fail("chdg_decode_device: null engine");
    return e->eng.decode(d_fields, field_stride, 0, nfields, frame_begin, frame_end, d_out, (cudaStream_t)stream);
}

int chdg_decode_host(chdg_engine *e, const uint16_t *h_fields, int64_t field_stride, int32_t nfields,
                     int32_t frame_begin, int32_t frame_end, void *h_out, void *stream)
{
    if (!e) return chdg::arg_fail("chdg_decode_host: null engine");
    return e->eng.decode_host(h_fields, field_stride, nfields, frame_begin, frame_end, h_out, (cudaStream_t)stream);
}

int chdg_engine_set_profiling(chdg_engine *e, int on)
{
    if (!e) return chdg::arg_fail("chdg_engine_set_profiling: null engine");
    e->eng.set_profiling(on != 0);
    e->eng.reset_kernel_times();
    return 0;
}

int chdg_engine_kernel_times(chdg_engine *e, double *ms_transform, double *ms_demod, int64_t *launches)
{
    if (!e) return chdg::arg_fail("chdg_engine_kernel_times: null engine");
    long long n = 0;
    const int rc = e->eng.kernel_times(ms_transform, ms_demod, &n);
    if (launches) *launches = n;
    return rc;
}

int chdg_chroma_device(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                       int32_t frame_begin, int32_t frame_end, float *d_chroma, void *stream)
{
    if (!e) return chdg::arg_fail("chdg_chroma_device: null engine");
    return e->eng.chroma(d_fields, field_stride, nfields, frame_begin, frame_end, d_chroma, (cudaStream_t)stream);
}

int chdg_engine_set_max_batch_frames(chdg_engine *e, int32_t frames)
{
    if (!e) return chdg::arg_fail("chdg_engine_set_max_batch_frames: null engine");
    if (frames < 1) return chdg::arg_fail("chdg_engine_set_max_batch_frames: frames must be at least 1");
    e->eng.set_max_batch_frames(frames);
    return 0;
}

int chdg_engine_set_tc_form(chdg_engine *e, int32_t variant)
{
    if (!e) return chdg::arg_fail("chdg_engine_set_tc_form: null engine");
    return e->eng.set_tc_form(variant);
}

int chdg_engine_set_masknet(chdg_engine *e, chdg_masknet *net)
{
    if (!e) return chdg::arg_fail("chdg_engine_set_masknet: null engine");
    return e->eng.set_masknet(net != nullptr ? chdg::masknet_of(net) : nullptr);
}

int chdg_engine_learned_stats(chdg_engine *e, int64_t *tiles, int64_t *fallback_tiles)
{
    if (!e) return chdg::arg_fail("chdg_engine_learned_stats: null engine");
    long long t = 0, f = 0;
    const int rc = e->eng.learned_stats(&t, &f);
    if (tiles) *tiles = t;
    if (fallback_tiles) *fallback_tiles = f;
    return rc;
}

int chdg_learned_features(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                          int32_t frame_begin, int32_t frame_end, uint16_t *d_feat, float *d_spec,
                          float *d_threshold_p, void *stream)
{
    if (!e) return chdg::arg_fail("chdg_learned_features: null engine");
    return e->eng.learned_features(d_fields, field_stride, nfields, frame_begin, frame_end, d_feat,
                                   reinterpret_cast<float2 *>(d_spec), d_threshold_p, (cudaStream_t)stream);
}

int chdg_learned_chroma(chdg_engine *e, const uint16_t *d_fields, int64_t field_stride, int32_t nfields,
                        int32_t frame_begin, int32_t frame_end, const float *d_p, const uint8_t *d_fallback,
                        float *d_chroma, void *stream)
{
    if (!e) return chdg::arg_fail("chdg_learned_chroma: null engine");
    return e->eng.learned_chroma(d_fields, field_stride, nfields, frame_begin, frame_end, d_p, d_fallback, d_chroma,
                                 (cudaStream_t)stream);
}

int chdg_engine_stats(chdg_engine *e, uint64_t *exact_decisions, uint64_t *fp32_flips)
{
    if (!e) return chdg::arg_fail("chdg_engine_stats: null engine");
    return e->eng.stats(exact_decisions, fp32_flips);
}

}  // extern "C"
#pragma GCC visibility pop
