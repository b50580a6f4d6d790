// abi_decoder.cpp -- decoder handles, options, commit and frame decode of the
// chd_* ABI (include/chromadec/decoder.h), following the reference's
// src/abi/c_api_decoder.cpp and src/decoders/registry.cpp. Options are
// stashed until commit and validated there in the reference's order, so the
// same calls fail with the same statuses; CHD_DEC_TRANSFORM_2D and
// CHD_DEC_TRANSFORM_3D then decode on the GPU through FramePipeline.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <thread>

#include <cuda_runtime.h>

#include "abi_handles.h"
#include "error_state.h"
#include "log_sink.h"

namespace chdg {

namespace {

// chd_decode_frame decodes ahead in batches of this many frames; the
// batches of chd_decode_frames_async are larger, so each launch fills the GPU
// several times over (a 32-frame 3D launch is 2.4 waves of tiles, a 64-frame
// one 4.9) while the first upload and the last download stay short.
constexpr int kSyncBatchFrames = 32;
constexpr int kAsyncBatchFrames = 64;

chd_status_t fail(chd_status_t s, const std::string &msg)
{
    chd::detail::set_last_error(msg);
    return s;
}

bool is_comb(chd_decoder_kind_t k)
{
    return k == CHD_DEC_NTSC_1D || k == CHD_DEC_NTSC_2D || k == CHD_DEC_NTSC_3D || k == CHD_DEC_NTSC_3D_NO_ADAPT ||
           k == CHD_DEC_NN_TRANSFORM3D;
}
bool is_pal(chd_decoder_kind_t k)
{
    return k == CHD_DEC_PAL_2D || k == CHD_DEC_TRANSFORM_2D || k == CHD_DEC_TRANSFORM_3D;
}
bool is_ldzeug(chd_decoder_kind_t k)
{
    return k == CHD_DEC_LDZEUG_COLOR_CNN || k == CHD_DEC_LDZEUG_LUMA_SEP || k == CHD_DEC_LDZEUG_LUMA_SEP_FRAME;
}
bool known_kind(chd_decoder_kind_t k)
{
    switch (k) {
    case CHD_DEC_MONO: case CHD_DEC_NTSC_1D: case CHD_DEC_NTSC_2D: case CHD_DEC_NTSC_3D:
    case CHD_DEC_NTSC_3D_NO_ADAPT: case CHD_DEC_PAL_2D: case CHD_DEC_TRANSFORM_2D: case CHD_DEC_TRANSFORM_3D:
    case CHD_DEC_NN_TRANSFORM3D: case CHD_DEC_LDZEUG_COLOR_CNN: case CHD_DEC_LDZEUG_LUMA_SEP:
    case CHD_DEC_LDZEUG_LUMA_SEP_FRAME: case CHD_DEC_SECAM: case CHD_DEC_HVD_2D: case CHD_DEC_HVD_3D:
        return true;
    default:
        return false;
    }
}

// registry::resolveAuto (registry.cpp:96-107).
chd_decoder_kind_t resolve_auto(chd_decoder_kind_t kind, int system)
{
    if (kind != CHD_DEC_AUTO) return kind;
    switch (system) {
    case SYS_NTSC: return CHD_DEC_NTSC_2D;
    case SYS_PAL:
    case SYS_PAL_M: return CHD_DEC_PAL_2D;
    case SYS_SECAM: return CHD_DEC_SECAM;
    }
    return CHD_DEC_AUTO;
}

// parseChdPixelFormat / parseOutputFormat (c_api_decoder.cpp:53-77).
bool parse_format(const std::string &n, chd_pixel_format_t &f)
{
    static const struct { const char *lo, *hi; chd_pixel_format_t f; } names[] = {
        {"yuv444p16", "YUV444P16", CHD_PIXEL_YUV444P16}, {"rgb48", "RGB48", CHD_PIXEL_RGB48},
        {"gray16", "GRAY16", CHD_PIXEL_GRAY16},          {"yuv444ps", "YUV444PS", CHD_PIXEL_YUV444PS},
        {"rgbs", "RGBS", CHD_PIXEL_RGBS},                {"grays", "GRAYS", CHD_PIXEL_GRAYS},
        {"yuv440p16", "YUV440P16", CHD_PIXEL_YUV440P16}, {"yuv440ps", "YUV440PS", CHD_PIXEL_YUV440PS},
    };
    for (const auto &x : names)
        if (n == x.lo || n == x.hi) {
            f = x.f;
            return true;
        }
    return false;
}

// parseClampMode (c_api_decoder.cpp:81-91).
int parse_clamp(const std::string &n)
{
    if (n == "none" || n == "NONE") return CHD_CLAMP_NONE;
    if (n == "legal_rgb_sdr" || n == "LEGAL_RGB_SDR") return CHD_CLAMP_LEGAL_RGB_SDR;
    if (n == "legal_rgb_hdr" || n == "LEGAL_RGB_HDR") return CHD_CLAMP_LEGAL_RGB_HDR;
    if (n == "legal_ycbcr_bt601" || n == "LEGAL_YCBCR_BT601") return CHD_CLAMP_LEGAL_YCBCR_BT601;
    return -1;
}

// readTransformThresholds (registry.cpp:85-92): whitespace-separated
// numbers; a missing or unreadable file gives an empty list.
std::vector<double> read_thresholds(const std::string &path)
{
    std::vector<double> out;
    std::ifstream in(path);
    if (!in.is_open()) return out;
    double v;
    while (in >> v) out.push_back(v);
    return out;
}

template <typename T>
chd_status_t set_option(chd_decoder_t *d, const char *name, OptType type, T value,
                        std::unordered_map<std::string, T> OptionMaps::*dst)
{
    if (d == nullptr || name == nullptr) return fail(CHD_E_INVALID_ARG, "chd_decoder_set_option: null argument");
    if (d->committed) return fail(CHD_E_INVALID_ARG, "chd_decoder_set_option: decoder already committed");
    if (!option_applies(d->kind, name, type))
        return fail(CHD_E_INVALID_ARG,
                    std::string("chd_decoder_set_option: option \"") + name + "\" not valid for this decoder kind");
    (d->options.*dst)[name] = std::move(value);
    return CHD_OK;
}

template <typename M, typename T>
T find_or(const M &m, const char *k, T def)
{
    auto it = m.find(k);
    return it == m.end() ? def : it->second;
}

DropoutSettings dropout_settings(const chd_decoder_t *d)
{
    DropoutSettings s;
    s.enabled = d->dropoutOptsSet && d->dropoutOpts.enabled != 0;
    s.overcorrect = d->dropoutOpts.overcorrect != 0;
    s.intra = d->dropoutOpts.intra_field_only != 0;
    return s;
}

// The settings a decode runs with: dropout_settings plus, when concealment
// is on, the video's extra sources. The first such decode freezes the
// extras and builds their alignment once (c_api_decoder.cpp:219-241).
DropoutSettings decode_dropout_settings(chd_decoder_t *d)
{
    DropoutSettings s = dropout_settings(d);
    if (!s.enabled) return s;
    chd_video_t *v = d->video;
    v->extrasFrozen.store(true, std::memory_order_release);
    if (v->extras.empty()) return s;
    std::lock_guard<std::mutex> l(d->sourcesMutex);
    if (!d->multiSource) {
        auto ms = std::make_shared<MultiSource>();
        std::vector<AlignedSource> all;
        all.push_back({&v->cap, d->firstFieldFirst()});
        for (const auto &x : v->extras) {
            const AlignedSource a{x.get(), x->isFirstFieldFirst() != d->reverseFieldOrder};
            all.push_back(a);
            ms->extras.push_back(a);
        }
        ms->alignment = SourceAlignment(std::move(all));
        d->multiSource = std::move(ms);
    }
    s.sources = d->multiSource;
    return s;
}

void publish_stats(chd_decoder_t *d, const FramePlan &p)
{
    std::lock_guard<std::mutex> l(d->statsMutex);
    d->lastDropoutStats.corrected = p.corrected;
    d->lastDropoutStats.failed = p.failed;
    d->lastDropoutStats.total_distance = p.totalDistance;
}

chd_status_t check_decodable(const chd_decoder_t *d, const char *caller)
{
    if (!d->committed) return fail(CHD_E_INVALID_ARG, std::string(caller) + ": chd_decoder_commit not called");
    if (d->resolvedKind == CHD_DEC_NONE)
        return fail(CHD_E_DECODER_INCOMPATIBLE,
                    std::string(caller) + ": decoder kind is CHD_DEC_NONE (geometry/dropout only)");
    return CHD_OK;
}

}  // namespace

bool option_applies(chd_decoder_kind_t kind, const std::string &name, OptType type)
{
    // output + pipeline-shape options apply to every kind (registry.cpp:47-66)
    if (type == OptType::I32 && (name == CHD_OPT_PADDING_MULTIPLE || name == CHD_OPT_THREAD_COUNT)) return true;
    if (type == OptType::Str && (name == CHD_OPT_OUTPUT_FORMAT || name == CHD_OPT_OUTPUT_CLAMP ||
                                 name == CHD_OPT_COLOR_DIFFERENCE_PRECISION ||
                                 name == CHD_OPT_BROADCAST_SCALING_PRECISION))
        return true;
    if (type == OptType::Bool && (name == CHD_OPT_OUTPUT_Y4M_HEADERS || name == CHD_OPT_REVERSE_FIELD_ORDER))
        return true;
    if (type == OptType::I32 && (name == CHD_OPT_FIRST_ACTIVE_FRAME_LINE || name == CHD_OPT_LAST_ACTIVE_FRAME_LINE ||
                                 name == CHD_OPT_FIRST_ACTIVE_SAMPLE || name == CHD_OPT_LAST_ACTIVE_SAMPLE))
        return true;
    const bool comb = is_comb(kind) || kind == CHD_DEC_AUTO;
    const bool pal = is_pal(kind) || kind == CHD_DEC_AUTO;
    const bool ldzeug = is_ldzeug(kind);
    const bool secam = kind == CHD_DEC_SECAM;
    const bool hvd = kind == CHD_DEC_HVD_2D || kind == CHD_DEC_HVD_3D;
    const bool tpal = kind == CHD_DEC_TRANSFORM_2D || kind == CHD_DEC_TRANSFORM_3D;
    if (type == OptType::F64) {
        if (name == CHD_OPT_CHROMA_GAIN) return comb || pal || ldzeug || secam || hvd;
        if (name == CHD_OPT_CHROMA_PHASE_DEG) return comb || pal || ldzeug || hvd;
        if (name == CHD_OPT_LUMA_NR_LEVEL) return comb || pal || kind == CHD_DEC_MONO;
        if (name == CHD_OPT_CHROMA_NR_LEVEL) return comb;
        if (name == CHD_OPT_COMB_ADAPT_THRESHOLD || name == CHD_OPT_COMB_CHROMA_WEIGHT) return kind == CHD_DEC_NTSC_3D;
        if (name == CHD_OPT_CHROMA_CLICK_NR_LEVEL || name == CHD_OPT_CHROMA_CLICK_ENV_DIP_DB ||
            name == CHD_OPT_CHROMA_CLICK_FREQ_OVERSHOOT)
            return secam;
        if (name == CHD_OPT_TRANSFORM_THRESHOLD) return tpal;
        if (name == CHD_OPT_HVD_TEMPORAL_STRENGTH) return kind == CHD_DEC_HVD_3D;
        if (name == CHD_OPT_NN_INPUT_MAGNITUDE_SCALE) return kind == CHD_DEC_NN_TRANSFORM3D;
    } else if (type == OptType::Bool) {
        if (name == CHD_OPT_PHASE_COMPENSATION) return comb || ldzeug;
        if (name == CHD_OPT_COMB_SHOW_MAP) return kind == CHD_DEC_NTSC_3D;
        if (name == CHD_OPT_NN_CHROMA_BANDPASS)
            return kind == CHD_DEC_LDZEUG_LUMA_SEP || kind == CHD_DEC_LDZEUG_LUMA_SEP_FRAME;
    } else if (type == OptType::Str) {
        if (name == CHD_OPT_CHROMA_IDENT_MODE || name == CHD_OPT_CHROMA_IDENT_MANUAL) return secam;
        if (name == CHD_OPT_TRANSFORM_THRESHOLDS_FILE) return tpal;
    } else if (type == OptType::I32) {
        if (name == CHD_OPT_HVD_CG_ITERATIONS) return hvd;
    }
    return false;
}

int make_pipeline(chd_decoder_t *d, std::unique_ptr<FramePipeline> &out, int batch_frames)
{
    if (cudaSetDevice(d->device) != cudaSuccess)
        return fail(CHD_E_INTERNAL, "chromadec_gb300: cannot select the decoder's CUDA device");
    auto p = std::make_unique<FramePipeline>();
    chdg_config c = d->cfg;
    c.thresholds = d->thresholds.empty() ? nullptr : d->thresholds.data();
    c.n_thresholds = (int32_t)d->thresholds.size();
    const int rc = p->init(&d->video->cap, d->geom, c, d->firstFieldFirst(), batch_frames);
    if (rc != CHD_OK) return rc;
    p->set_dropout(dropout_settings(d));
    out = std::move(p);
    return CHD_OK;
}

chd_frame_t *make_frame(chd_decoder_t *d, const std::shared_ptr<HostChunk> &chunk, size_t offset, int64_t index)
{
    auto *f = new chd_frame();
    f->format = d->outputPixelFormat;
    f->width = d->outWidth;
    f->height = d->outHeight;
    f->chunk = chunk;
    f->pixels = static_cast<const char *>(chunk->data) + offset;
    f->info.format = f->format;
    f->info.width = f->width;
    f->info.height = f->height;
    f->info.num_planes = (f->format == CHD_PIXEL_GRAY16 || f->format == CHD_PIXEL_GRAYS) ? 1 : 3;
    f->info.frame_index = index;
    return f;
}

}  // namespace chdg

using namespace chdg;

// ---- lifecycle and options (c_api_decoder.cpp:533-604) ----------------------

CHD_API chd_status_t chd_decoder_create(chd_video_t *v, chd_decoder_kind_t kind, chd_decoder_t **out)
{
    if (v == nullptr || out == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_create: null argument");
    auto d = std::make_unique<chd_decoder>();
    d->video = v;
    d->kind = kind;
    *out = d.release();
    return CHD_OK;
}

CHD_API void chd_decoder_free(chd_decoder_t *d)
{
    if (d == nullptr) return;
    d->ahead.clear();
    delete d;
}

CHD_API chd_status_t chd_decoder_set_option_f64(chd_decoder_t *d, const char *name, double v)
{
    return set_option(d, name, OptType::F64, v, &OptionMaps::f64);
}

CHD_API chd_status_t chd_decoder_set_option_i32(chd_decoder_t *d, const char *name, int32_t v)
{
    return set_option(d, name, OptType::I32, v, &OptionMaps::i32);
}

CHD_API chd_status_t chd_decoder_set_option_bool(chd_decoder_t *d, const char *name, int v)
{
    return set_option<bool>(d, name, OptType::Bool, v != 0, &OptionMaps::boolean);
}

CHD_API chd_status_t chd_decoder_set_option_str(chd_decoder_t *d, const char *name, const char *v)
{
    if (v == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_set_option_str: null argument (value)");
    return set_option<std::string>(d, name, OptType::Str, v, &OptionMaps::str);
}

CHD_API chd_status_t chd_decoder_has_option(const chd_decoder_t *d, const char *name)
{
    if (d == nullptr || name == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_has_option: null argument");
    for (OptType t : {OptType::F64, OptType::I32, OptType::Bool, OptType::Str})
        if (option_applies(d->kind, name, t)) return CHD_OK;
    return CHD_E_INVALID_ARG;
}

// No NN kinds in this library: the reference's answer when built without NN
// support (c_api_decoder.cpp:581-600).
CHD_API chd_status_t chd_decoder_set_nn_model(chd_decoder_t *d, chd_nn_model_t *)
{
    if (d == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_set_nn_model: null argument");
    if (d->committed) return fail(CHD_E_INVALID_ARG, "chd_decoder_set_nn_model: decoder already committed");
    return fail(CHD_E_INTERNAL, "chd_decoder_set_nn_model: library built without NN support");
}

CHD_API chd_status_t chd_decoder_get_chroma_click_thresholds(const chd_decoder_t *d, double *env, double *freq)
{
    if (d == nullptr || env == nullptr || freq == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_get_chroma_click_thresholds: null argument");
    return fail(CHD_E_UNSUPPORTED, "chd_decoder_get_chroma_click_thresholds: no decode has run with "
                                   "chroma_click_nr_level > 0");
}

// ---- commit (c_api_decoder.cpp:604-1022) -------------------------------------

CHD_API chd_status_t chd_decoder_commit(chd_decoder_t *d)
{
    if (d == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_commit: null argument");
    if (d->committed) return CHD_OK;
    if (d->video == nullptr) return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: video has no source");
    const OptionMaps &o = d->options;
    const VideoParams &src = d->video->cap.vp();
    const chd_decoder_kind_t resolved = resolve_auto(d->kind, src.system);

    const int32_t padding = find_or(o.i32, CHD_OPT_PADDING_MULTIPLE, 1);
    if (padding < 1 || padding > 1024)
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: padding_multiple must be between 1 (no padding) and 1024");
    const bool y4m = find_or(o.boolean, CHD_OPT_OUTPUT_Y4M_HEADERS, false);

    chd_pixel_format_t fmt = CHD_PIXEL_YUV444P16;
    if (auto it = o.str.find(CHD_OPT_OUTPUT_FORMAT); it != o.str.end() && !parse_format(it->second, fmt))
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: unknown output_format \"" + it->second + "\"");
    int clamp = CHD_CLAMP_NONE;
    if (auto it = o.str.find(CHD_OPT_OUTPUT_CLAMP); it != o.str.end() && (clamp = parse_clamp(it->second)) < 0)
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: unknown output_clamp \"" + it->second + "\"");
    // ColorConversion (src/common/color_conversion.cpp:33-81)
    double kr = 0.299, kb = 0.114, uRed = 0.49211104112248356308804691718185, vRed = 0.87728321993817866838972487283129;
    if (auto it = o.str.find(CHD_OPT_COLOR_DIFFERENCE_PRECISION); it != o.str.end()) {
        if (it->second == "classic") kr = 0.30, kb = 0.11;
        else if (it->second != "modern")
            return fail(CHD_E_INVALID_ARG,
                        "chd_decoder_commit: unknown color_difference_precision \"" + it->second + "\"");
    }
    if (auto it = o.str.find(CHD_OPT_BROADCAST_SCALING_PRECISION); it != o.str.end()) {
        if (it->second == "classic") uRed = 0.493, vRed = 0.877;
        else if (it->second == "modern") uRed = 0.492111, vRed = 0.877283;
        else if (it->second != "scientific")
            return fail(CHD_E_INVALID_ARG,
                        "chd_decoder_commit: unknown broadcast_scaling_precision \"" + it->second + "\"");
    }
    {
        const bool is440 = fmt == CHD_PIXEL_YUV440P16 || fmt == CHD_PIXEL_YUV440PS;
        const bool lumaOnly = fmt == CHD_PIXEL_GRAY16 || fmt == CHD_PIXEL_GRAYS;
        if (src.system == SYS_SECAM && !is440 && !lumaOnly)
            return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: SECAM sources decode to 4:4:0 chroma "
                                           "(\"yuv440ps\"/\"yuv440p16\") or luma-only (\"grays\"/\"gray16\"); "
                                           "vertical chroma reconstruction is the consumer's choice");
        if (is440 && src.system != SYS_SECAM)
            return fail(CHD_E_INVALID_ARG,
                        "chd_decoder_commit: 4:4:0 output is produced only by line-sequential (SECAM) decodes");
        if (is440 && y4m)
            return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: output_y4m_headers does not support 4:4:0 output");
    }
    {
        const auto mode = o.str.find(CHD_OPT_CHROMA_IDENT_MODE), manual = o.str.find(CHD_OPT_CHROMA_IDENT_MANUAL);
        std::string m;
        if (mode != o.str.end()) {
            m = mode->second;
            if (m != "auto" && m != "porch" && m != "bottles" && m != "manual")
                return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: unknown chroma_ident_mode \"" + m + "\"");
        }
        if (manual != o.str.end()) {
            if (manual->second != "db_first" && manual->second != "dr_first")
                return fail(CHD_E_INVALID_ARG,
                            "chd_decoder_commit: unknown chroma_ident_manual \"" + manual->second + "\"");
            if (m != "manual")
                return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: chroma_ident_manual is only meaningful with "
                                               "chroma_ident_mode=\"manual\"");
        } else if (m == "manual") {
            return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: chroma_ident_mode=\"manual\" requires "
                                           "chroma_ident_manual (\"db_first\" or \"dr_first\")");
        }
    }
    {
        const auto lvl = o.f64.find(CHD_OPT_CHROMA_CLICK_NR_LEVEL);
        const double level = lvl != o.f64.end() ? lvl->second : 1.0;
        if (lvl != o.f64.end() && (!std::isfinite(level) || level < 0.0 || level > 1.0))
            return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: chroma_click_nr_level must be in [0.0, 1.0]");
        for (const char *name : {CHD_OPT_CHROMA_CLICK_ENV_DIP_DB, CHD_OPT_CHROMA_CLICK_FREQ_OVERSHOOT}) {
            auto it = o.f64.find(name);
            if (it == o.f64.end()) continue;
            if (!std::isfinite(it->second) || it->second <= 0.0)
                return fail(CHD_E_INVALID_ARG, std::string("chd_decoder_commit: ") + name + " must be a positive threshold");
            if (level <= 0.0)
                return fail(CHD_E_INVALID_ARG, std::string("chd_decoder_commit: ") + name +
                                                   " is only meaningful when chroma_click_nr_level > 0");
        }
    }
    if (auto it = o.f64.find(CHD_OPT_NN_INPUT_MAGNITUDE_SCALE);
        it != o.f64.end() && (!std::isfinite(it->second) || it->second <= 0.0))
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: nn_input_magnitude_scale must be finite and > 0");
    if (auto it = o.i32.find(CHD_OPT_HVD_CG_ITERATIONS); it != o.i32.end() && it->second < 0)
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: hvd_cg_iterations must be >= 0 "
                                       "(0 decodes with the holographic init alone)");
    if (auto it = o.f64.find(CHD_OPT_HVD_TEMPORAL_STRENGTH);
        it != o.f64.end() && (!std::isfinite(it->second) || it->second < 0.0))
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: hvd_temporal_strength must be >= 0 "
                                       "(0 adapts to the measured Y/C ambiguity)");

    // active crop: applyCropOverrides + validateCrop (c_api_decoder.cpp:93-137)
    VideoParams vp = src;
    if (auto it = o.i32.find(CHD_OPT_FIRST_ACTIVE_FRAME_LINE); it != o.i32.end()) vp.firstActiveFrameLine = it->second;
    if (auto it = o.i32.find(CHD_OPT_LAST_ACTIVE_FRAME_LINE); it != o.i32.end()) vp.lastActiveFrameLine = it->second;
    if (auto it = o.i32.find(CHD_OPT_FIRST_ACTIVE_SAMPLE); it != o.i32.end()) vp.activeVideoStart = it->second;
    if (auto it = o.i32.find(CHD_OPT_LAST_ACTIVE_SAMPLE); it != o.i32.end()) vp.activeVideoEnd = it->second + 1;
    if (vp.activeVideoStart < 0 || vp.activeVideoEnd > vp.fieldWidth || vp.activeVideoEnd <= vp.activeVideoStart)
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: active sample crop must satisfy 0 <= first_active_sample "
                                       "<= last_active_sample < field_width");
    if (vp.firstActiveFrameLine < 0 || vp.lastActiveFrameLine >= vp.fieldHeight * 2 - 1 ||
        vp.lastActiveFrameLine < vp.firstActiveFrameLine)
        return fail(CHD_E_INVALID_ARG, "chd_decoder_commit: active frame-line crop must satisfy 0 <= "
                                       "first_active_frame_line <= last_active_frame_line < (2 * field_height) - 1");
    const bool reverse = find_or(o.boolean, CHD_OPT_REVERSE_FIELD_ORDER, false);

    // geometry and output framing (OutputWriter::updateConfiguration)
    chdg_geometry g{};
    g.field_width = vp.fieldWidth;
    g.field_height = vp.fieldHeight;
    g.active_start = vp.activeVideoStart;
    g.active_end = vp.activeVideoEnd;
    g.first_active_frame_line = vp.firstActiveFrameLine;
    g.last_active_frame_line = vp.lastActiveFrameLine;
    g.burst_start = vp.colourBurstStart;
    g.burst_end = vp.colourBurstEnd;
    g.black = vp.black16bIre;
    g.white = vp.white16bIre;
    g.sample_rate = vp.sampleRate;
    g.fsc = vp.fSC;
    int w = 0, h = 0, lp = 0, tp = 0;
    output_geometry(g, padding, w, h, lp, tp);

    chdg_config c{};
    chdg_default_config(&c, (int32_t)resolved);
    c.clamp_mode = clamp;
    c.padding_multiple = padding;
    c.kr = kr;
    c.kb = kb;
    c.u_reduction = uRed;
    c.v_reduction = vRed;
    c.ecb_from_u = 1.0 / ((2.0 * (1.0 - kb)) * uRed);
    c.ecr_from_v = 1.0 / ((2.0 * (1.0 - kr)) * vRed);

    auto snapshot = [&]() {
        d->resolvedKind = resolved;
        d->reverseFieldOrder = reverse;
        d->outputPixelFormat = fmt;
        d->geom = g;
        d->framing = {vp.activeVideoStart, vp.activeVideoEnd - vp.activeVideoStart, w, h, vp.firstActiveFrameLine,
                      lp, tp, vp.fieldWidth};
        d->outWidth = w;
        d->outHeight = h;
        d->numFrames = d->video->cap.numFrames(d->video->cap.isFirstFieldFirst() != reverse);
    };

    if (d->kind == CHD_DEC_NONE) {   // geometry / dropout queries only
        snapshot();
        d->threadCount = 0;
        d->committed = true;
        return CHD_OK;
    }
    int32_t threads = find_or(o.i32, CHD_OPT_THREAD_COUNT, 0);
    if (threads <= 0) {
        const unsigned hc = std::thread::hardware_concurrency();
        threads = hc == 0 ? 2 : (int32_t)hc;
    }
    if (!known_kind(resolved))
        return fail(CHD_E_DECODER_UNKNOWN, "chd_decoder_commit: unknown or unsupported decoder kind");
    if (resolved != CHD_DEC_PAL_2D && resolved != CHD_DEC_TRANSFORM_2D && resolved != CHD_DEC_TRANSFORM_3D)
        return fail(CHD_E_UNSUPPORTED, "chd_decoder_commit: this library decodes CHD_DEC_PAL_2D, "
                                       "CHD_DEC_TRANSFORM_2D and CHD_DEC_TRANSFORM_3D only");
    // PalDecoder::configure (src/decoders/palcolour/pal_decoder.cpp:38-43)
    if (src.system != SYS_PAL && src.system != SYS_PAL_M) {
        log_returned(CHD_LOG_ERROR, "This decoder is for PAL video sources only");
        return fail(CHD_E_DECODER_INCOMPATIBLE, "chd_decoder_commit: This decoder is for PAL video sources only");
    }
    c.threshold = find_or(o.f64, CHD_OPT_TRANSFORM_THRESHOLD, c.threshold);
    c.chroma_gain = find_or(o.f64, CHD_OPT_CHROMA_GAIN, c.chroma_gain);
    c.chroma_phase_deg = find_or(o.f64, CHD_OPT_CHROMA_PHASE_DEG, c.chroma_phase_deg);
    // doYNR runs only for yNRLevel > 0.0 (palcolour.cpp:644-646); anything else is off
    c.y_nr_level = std::max(0.0, find_or(o.f64, CHD_OPT_LUMA_NR_LEVEL, 0.0));
    c.output_format = (int32_t)fmt;   // chd_pixel_format_t 0..5 (4:4:0 was rejected above)
    std::vector<double> thr;
    if (auto it = o.str.find(CHD_OPT_TRANSFORM_THRESHOLDS_FILE);
        resolved != CHD_DEC_PAL_2D && it != o.str.end() && !it->second.empty()) {
        thr = read_thresholds(it->second);
        const size_t need = resolved == CHD_DEC_TRANSFORM_2D ? 80 : 768;
        // TransformPal::updateConfiguration asserts this count (transform_pal.cpp:62-72)
        if (!thr.empty() && thr.size() != need)
            return fail(CHD_E_DECODER_INCOMPATIBLE, "chd_decoder_commit: transform_thresholds_file holds " +
                                                        std::to_string(thr.size()) + " values, this kind needs " +
                                                        std::to_string(need));
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return fail(CHD_E_INTERNAL, "chd_decoder_commit: no CUDA device is available");
    }
    snapshot();
    d->cfg = c;
    d->thresholds = std::move(thr);
    d->threadCount = threads;
    d->device = dev;
    std::unique_ptr<FramePipeline> p;
    if (const int rc = make_pipeline(d, p, kSyncBatchFrames); rc != CHD_OK) {
        chd::detail::set_last_error("chd_decoder_commit: " + chd::detail::get_last_error());
        return (chd_status_t)(rc == CHD_E_INVALID_ARG ? CHD_E_DECODER_INCOMPATIBLE : rc);
    }
    d->syncPipe = std::move(p);
    d->committed = true;
    return CHD_OK;
}

// ---- decode (c_api_decoder.cpp:1063-1152) ------------------------------------

CHD_API chd_status_t chd_decode_frame(chd_decoder_t *d, int64_t frame_index, chd_frame_t **out)
{
    if (d == nullptr || out == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decode_frame: null argument");
    *out = nullptr;
    if (const chd_status_t s = check_decodable(d, "chd_decode_frame"); s != CHD_OK) return s;
    std::lock_guard<std::mutex> lock(d->syncMutex);
    if (frame_index < 0 || frame_index >= d->numFrames)
        return fail(CHD_E_OUT_OF_RANGE, "chd_decode_frame: frame_index out of range");
    const uint64_t rev = d->dropoutRevision.load(std::memory_order_acquire);
    auto it = d->ahead.find(frame_index);
    if (it == d->ahead.end() || it->second.revision != rev) {
        // Decode ahead while requests run in order; a jump decodes one frame.
        d->ahead.clear();
        const int64_t n = (frame_index == d->lastIndex + 1) ? kSyncBatchFrames : 1;
        const int64_t end = std::min<int64_t>(d->numFrames, frame_index + n);
        FramePipeline &p = *d->syncPipe;
        cudaSetDevice(d->device);
        p.set_dropout(decode_dropout_settings(d));
        const size_t fb = p.frame_bytes();
        const int rc = p.decode(
            frame_index, end,
            [&](const std::shared_ptr<HostChunk> &chunk, int64_t first, int count) {
                for (int i = 0; i < count; i++) {
                    CachedFrame cf;
                    cf.chunk = chunk;
                    cf.offset = fb * (size_t)i;
                    cf.stats = p.frame_stats(first + i);
                    cf.revision = rev;
                    d->ahead[first + i] = std::move(cf);
                }
            },
            nullptr, nullptr);
        if (rc != CHD_OK) {
            d->ahead.clear();
            chd::detail::set_last_error("chd_decode_frame: " + chd::detail::get_last_error());
            return (chd_status_t)rc;
        }
        it = d->ahead.find(frame_index);
        if (it == d->ahead.end()) return fail(CHD_E_INTERNAL, "chd_decode_frame: frame was not produced");
    }
    CachedFrame cf = std::move(it->second);
    d->ahead.erase(d->ahead.begin(), std::next(it));
    d->lastIndex = frame_index;
    publish_stats(d, cf.stats);
    *out = make_frame(d, cf.chunk, cf.offset, frame_index);
    return CHD_OK;
}

CHD_API chd_status_t chd_decode_frames_async(chd_decoder_t *d, const int64_t *indices, size_t n, chd_frame_done_cb cb,
                                             void *user, chd_cancel_t *cancel)
{
    if (d == nullptr || cb == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_decode_frames_async: null argument");
    if (n > 0 && indices == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_decode_frames_async: null argument (indices)");
    if (const chd_status_t s = check_decodable(d, "chd_decode_frames_async"); s != CHD_OK) return s;
    if (n == 0) return CHD_OK;

    // A pipeline of its own for this call: concurrent calls, and calls made
    // from inside a callback, never share one.
    std::unique_ptr<FramePipeline> pipe;
    {
        std::lock_guard<std::mutex> l(d->poolMutex);
        if (!d->pool.empty()) {
            pipe = std::move(d->pool.back());
            d->pool.pop_back();
        }
    }
    chd_status_t failure = CHD_OK;
    std::string failureDetail;
    if (!pipe) {
        failure = (chd_status_t)make_pipeline(d, pipe, kAsyncBatchFrames);
        failureDetail = chd::detail::get_last_error();
    }

    // Requests sorted by frame; out-of-range ones answered first.
    std::vector<std::pair<int64_t, size_t>> order;
    order.reserve(n);
    for (size_t i = 0; i < n; i++) {
        if (indices[i] < 0 || indices[i] >= d->numFrames) {
            chd::detail::set_last_error("chd_decode_frame: frame_index out of range");
            cb(user, CHD_E_OUT_OF_RANGE, indices[i], nullptr);
        } else {
            order.emplace_back(indices[i], i);
        }
    }
    std::sort(order.begin(), order.end());
    std::vector<bool> done(order.size(), false);
    auto is_cancelled = [cancel]() { return cancel != nullptr && cancel->requested.load(std::memory_order_acquire); };

    if (failure == CHD_OK) {
        cudaSetDevice(d->device);
        pipe->set_dropout(decode_dropout_settings(d));
        const size_t fb = pipe->frame_bytes();
        size_t k = 0;
        while (k < order.size() && failure == CHD_OK && !is_cancelled()) {
            // one run of consecutive frames
            size_t e = k + 1;
            while (e < order.size() && order[e].first <= order[e - 1].first + 1) e++;
            const int64_t a = order[k].first, b = order[e - 1].first + 1;
            size_t cursor = k;
            const int rc = pipe->decode(
                a, b,
                [&](const std::shared_ptr<HostChunk> &chunk, int64_t first, int count) {
                    while (cursor < e && order[cursor].first < first + count) {
                        const int64_t f = order[cursor].first;
                        // a request made after cancellation is answered CHD_E_CANCELLED below
                        if (f >= first && !is_cancelled()) {
                            publish_stats(d, pipe->frame_stats(f));
                            done[cursor] = true;
                            cb(user, CHD_OK, f, make_frame(d, chunk, fb * (size_t)(f - first), f));
                        }
                        cursor++;
                    }
                },
                is_cancelled, nullptr);
            if (rc != CHD_OK) {
                failure = (chd_status_t)rc;
                failureDetail = chd::detail::get_last_error();
            }
            k = e;
        }
    }
    // Everything not delivered: cancelled, or the failure that stopped the run.
    for (size_t i = 0; i < order.size(); i++) {
        if (done[i]) continue;
        if (failure != CHD_OK) {
            chd::detail::set_last_error("chd_decode_frames_async: " + failureDetail);
            cb(user, failure, order[i].first, nullptr);
        } else {
            cb(user, CHD_E_CANCELLED, order[i].first, nullptr);
        }
    }
    if (pipe) {
        std::lock_guard<std::mutex> l(d->poolMutex);
        if (d->pool.size() < 2) d->pool.push_back(std::move(pipe));
    }
    return CHD_OK;
}

// ---- concealed fields (no counterpart in the reference ABI) ---------------

CHD_API int chdg_decoder_concealed_fields(chd_decoder_t *d, int64_t frame_index, uint16_t *out)
{
    if (d == nullptr || out == nullptr) return fail(CHD_E_INVALID_ARG, "chdg_decoder_concealed_fields: null argument");
    if (const chd_status_t s = check_decodable(d, "chdg_decoder_concealed_fields"); s != CHD_OK) return s;
    std::lock_guard<std::mutex> lock(d->syncMutex);
    if (frame_index < 0 || frame_index >= d->numFrames)
        return fail(CHD_E_OUT_OF_RANGE, "chdg_decoder_concealed_fields: frame_index out of range");
    cudaSetDevice(d->device);
    FramePipeline &p = *d->syncPipe;
    p.set_dropout(decode_dropout_settings(d));
    const int rc = p.conceal_frame(frame_index, out);
    if (rc != CHD_OK) {
        if (rc != CHD_E_OUT_OF_RANGE)
            chd::detail::set_last_error("chdg_decoder_concealed_fields: " + chd::detail::get_last_error());
        return rc;
    }
    return CHD_OK;
}
