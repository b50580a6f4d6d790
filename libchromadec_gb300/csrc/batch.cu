// batch.cu -- many captures of uneven length and mixed 2D/3D modes decoded
// together: chdg_batch_* (include/chromadec_gb300.h; no reference
// counterpart -- the reference decodes one capture per decoder).
//
// Layout. Each mode's captures share one frame index space, and a table
// gives every field's first sample in the caller's own buffers: the fields
// are read in place, never copied. In the 3D space every capture is preceded
// and followed by 3 frames of black fields (null table entries). Those gaps
// make the batch decode exactly the per-capture decode: the reference pads
// every 3D window with black outside the capture
// (src/decoders/source_field.cpp:88-170) and a frame's Z tiles reach 2 frames
// back and 3 ahead, so no tile of a capture's frame sees another capture. The
// 2D space has no gaps (its frames are independent). Per frame, a table holds
// the squared threshold of the capture that owns it (gap frames take the next
// capture's: their tiles feed that capture's first frames) and a table the
// frame's output pointer (null for gap frames, which are not written). One
// transform launch and one demodulator launch then cover every capture of a
// mode, so short captures no longer leave the GPU mostly idle.
//
// Dropouts. A capture with CHDG_CONCEAL set is copied once per decode into a
// device pool (the caller's fields stay as they are, so a replayed decode
// conceals the same samples again) and each of its frames with dropouts is
// concealed there by the pipeline's own kernel, from the plan the host makes
// once per batch shape (dropout_plan.cpp, DropoutCorrector::correctFrame);
// its field-table entries then point into the pool. A frame's plan reads only
// its own two fields, so concealing every frame once is what the reference's
// per-window concealment gives each window. Dropout masks (the detected
// mode's spans in output framing, c_api_dropout_detect.cpp:92-174) are
// rastered by one launch over every span of the batch.
//
// Graphs. The first decode of a batch shape runs eagerly (it sizes every
// buffer); the copies and launches of a shape are then captured once into a
// CUDA graph, and later decodes of the same captures replay it with one
// launch. chdg_batch_autotune times the schedule candidates (frames per work
// item, persistent or full grid) on the caller's batch and keeps the fastest.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "dropout_plan.h"
#include "engine.h"
#include "error_state.h"

namespace chdg {
int dropout_apply(uint16_t *fields, long long field_stride, int fw, const int *d_frames, const DropOp *d_ops,
                  const int *d_op_begin, int nframes, const uint16_t *extras, bool ntsc_taps, cudaStream_t s);
}

namespace {

constexpr int kGapFrames = 3;

int bfail(const std::string &m, int code = CHDG_E_INVALID_ARG)
{
    chd::detail::set_last_error("chromadec_gb300: " + m);
    return code;
}

int cfail(const char *what, cudaError_t e)
{
    cudaGetLastError();
    chd::detail::set_last_error(std::string("chromadec_gb300: ") + what + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? CHDG_E_OOM : CHDG_E_CUDA;
}

// One mode's share of a batch: its frame index space and the tables over it.
struct ModeLayout {
    std::vector<int> caps;               // capture indices of this mode
    std::vector<int64_t> first_frame;    // per listed capture: its first frame in the space
    int64_t frames = 0;                  // frames in the space (gaps included)
    std::vector<const uint16_t *> fptr;  // 2 per frame (null: black)
    std::vector<float> t2;               // 3 per frame
    std::vector<void *> outs;            // per frame
};

// A mask span of the batch: row `row` (a plane row's first sample) gets
// 0xFFFF in [x0, x1).
struct MaskSpan {
    uint16_t *row;
    int32_t x0, x1;
};

__global__ void batch_mask_kernel(const MaskSpan *spans)
{
    const MaskSpan m = spans[blockIdx.x];
    for (int x = m.x0 + (int)threadIdx.x; x < m.x1; x += blockDim.x) m.row[x] = 0xFFFF;
}

// Concealment of a batch: captures copied into the pool, the frames' plans.
struct ConcealPlan {
    struct Copy {
        const uint16_t *src;
        int64_t src_stride;
        int64_t pool_field;   // first pool field
        int32_t nfields;
    };
    std::vector<Copy> copies;
    std::vector<int> frames;        // per planned frame: its slot-0 pool field
    std::vector<int> op_begin;      // per planned frame, plus the end
    std::vector<chdg::DropOp> ops;
    std::vector<MaskSpan> spans;
    struct Clear {
        uint16_t *plane;
        size_t bytes;
    };
    std::vector<Clear> clears;      // mask buffers to zero
    int64_t pool_fields = 0;
};

// The device copy of one mode's tables.
struct ModeTables {
    const uint16_t **fptr = nullptr;
    float *t2 = nullptr;
    void **outs = nullptr;
    size_t cap = 0;   // frames

    ~ModeTables()
    {
        cudaFree(fptr);
        cudaFree(t2);
        cudaFree(outs);
    }
};

}  // namespace

struct chdg_batch {
    chdg_geometry g{};
    chdg_config c{};
    chdg::Engine eng3, eng2;
    ModeTables tab3, tab2;
    // concealment and masks of the current shape
    ConcealPlan cp;
    uint16_t *pool = nullptr;
    int64_t pool_cap = 0;     // fields
    int64_t pool_stride = 0;  // samples per pool field
    chdg::DropOp *d_ops = nullptr;
    int *d_idx = nullptr;     // frames, then op_begin
    MaskSpan *d_spans = nullptr;
    size_t ops_cap = 0, idx_cap = 0, spans_cap = 0;
    // the shape of the last decode, and its graph
    std::vector<chdg_capture> last;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int eager_runs = 0;

    ~chdg_batch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        cudaFree(pool);
        cudaFree(d_ops);
        cudaFree(d_idx);
        cudaFree(d_spans);
    }

    // VideoParameters of the batch's raster for the concealment planner
    chdg::VideoParams video_params() const
    {
        chdg::VideoParams vp;
        vp.system = g.field_height == 263 ? chdg::SYS_PAL_M : chdg::SYS_PAL;
        vp.fieldWidth = g.field_width;
        vp.fieldHeight = g.field_height;
        vp.sampleRate = g.sample_rate;
        vp.fSC = g.fsc;
        vp.activeVideoStart = g.active_start;
        vp.activeVideoEnd = g.active_end;
        vp.colourBurstStart = g.burst_start;
        vp.colourBurstEnd = g.burst_end;
        vp.black16bIre = g.black;
        vp.white16bIre = g.white;
        vp.blanking16bIre = g.black;
        vp.firstActiveFrameLine = g.first_active_frame_line;
        vp.lastActiveFrameLine = g.last_active_frame_line;
        return vp;
    }

    // Plans, pool placement and mask spans of the captures with dropouts;
    // `fields_of` gives each capture's field pointers (pool or caller).
    int plan_dropouts(const chdg_capture *caps, int n, std::vector<int64_t> &pool_first)
    {
        cp = ConcealPlan{};
        pool_first.assign((size_t)n, -1);
        const chdg::VideoParams vp = video_params();
        const int aw = g.active_end - g.active_start;
        const int ah = g.last_active_frame_line - g.first_active_frame_line + 1;
        const chdg::OutputFraming fr{g.active_start, aw, aw, ah, g.first_active_frame_line, 0, 0, g.field_width};
        const size_t plane = (size_t)aw * ah;
        for (int i = 0; i < n; i++) {
            const chdg_capture &k = caps[i];
            if (k.ndropouts < 0 || (k.ndropouts > 0 && k.dropouts == nullptr))
                return bfail("chdg_batch_decode: capture " + std::to_string(i) + " has a bad dropout list");
            const int nf = k.nfields / 2;
            std::vector<chdg::FieldMeta> meta((size_t)2 * nf);
            for (int f = 0; f < 2 * nf; f++) meta[f].isFirstField = (f & 1) == 0;
            for (int j = 0; j < k.ndropouts; j++) {
                const chdg_dropout &d = k.dropouts[j];
                if (d.field >= 0 && d.field < 2 * nf) meta[d.field].dropouts.push_back({d.startx, d.endx, d.field_line});
            }
            if (k.mask_out != nullptr) {
                cp.clears.push_back({k.mask_out, plane * sizeof(uint16_t) * (size_t)nf});
                for (int f = 0; f < nf; f++) {
                    if (meta[2 * f].dropouts.empty() && meta[2 * f + 1].dropouts.empty()) continue;
                    const std::vector<chdg::Span> sp = chdg::frame_spans(fr, meta[2 * f], true, meta[2 * f + 1], false,
                                                                         false);
                    for (const chdg::Span &s : sp)
                        cp.spans.push_back({k.mask_out + plane * (size_t)f + (size_t)s.y * aw, s.x_start, s.x_end});
                }
            }
            if ((k.conceal & CHDG_CONCEAL) == 0 || k.ndropouts == 0 || nf == 0) continue;
            pool_first[i] = cp.pool_fields;
            cp.copies.push_back({k.fields, k.field_stride, cp.pool_fields, 2 * nf});
            const bool oc = (k.conceal & CHDG_CONCEAL_OVERCORRECT) != 0, intra = (k.conceal & CHDG_CONCEAL_INTRA) != 0;
            for (int f = 0; f < nf; f++) {
                if (meta[2 * f].dropouts.empty() && meta[2 * f + 1].dropouts.empty()) continue;
                const chdg::FramePlan pl = chdg::plan_frame(vp, meta[2 * f], meta[2 * f + 1], oc, intra);
                if (pl.ops.empty()) continue;
                cp.frames.push_back((int)(cp.pool_fields + 2 * f));
                cp.op_begin.push_back((int)cp.ops.size());
                cp.ops.insert(cp.ops.end(), pl.ops.begin(), pl.ops.end());
            }
            cp.pool_fields += 2 * nf;
        }
        cp.op_begin.push_back((int)cp.ops.size());
        return 0;
    }

    int upload_dropouts(cudaStream_t s)
    {
        cudaError_t e;
        pool_stride = ((int64_t)g.field_width * g.field_height + 63) & ~(int64_t)63;
        if (cp.pool_fields > pool_cap) {
            cudaFree(pool);
            pool = nullptr;
            pool_cap = 0;
            if ((e = cudaMalloc(&pool, (size_t)cp.pool_fields * pool_stride * sizeof(uint16_t))) != cudaSuccess)
                return cfail("concealment pool", e);
            pool_cap = cp.pool_fields;
        }
        auto grow = [&](void **p, size_t &cap, size_t need, size_t elem) -> cudaError_t {
            if (need <= cap) return cudaSuccess;
            cudaFree(*p);
            *p = nullptr;
            cap = 0;
            const cudaError_t r = cudaMalloc(p, need * elem);
            if (r == cudaSuccess) cap = need;
            return r;
        };
        const size_t nidx = cp.frames.size() + cp.op_begin.size();
        if ((e = grow((void **)&d_ops, ops_cap, std::max<size_t>(cp.ops.size(), 1), sizeof(chdg::DropOp))) !=
                cudaSuccess ||
            (e = grow((void **)&d_idx, idx_cap, std::max<size_t>(nidx, 1), sizeof(int))) != cudaSuccess ||
            (e = grow((void **)&d_spans, spans_cap, std::max<size_t>(cp.spans.size(), 1), sizeof(MaskSpan))) !=
                cudaSuccess)
            return cfail("concealment tables", e);
        std::vector<int> idx(cp.frames);
        idx.insert(idx.end(), cp.op_begin.begin(), cp.op_begin.end());
        if (!cp.ops.empty() &&
            (e = cudaMemcpyAsync(d_ops, cp.ops.data(), cp.ops.size() * sizeof(chdg::DropOp), cudaMemcpyHostToDevice,
                                 s)) != cudaSuccess)
            return cfail("concealment tables", e);
        if ((e = cudaMemcpyAsync(d_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, s)) !=
            cudaSuccess)
            return cfail("concealment tables", e);
        if (!cp.spans.empty() &&
            (e = cudaMemcpyAsync(d_spans, cp.spans.data(), cp.spans.size() * sizeof(MaskSpan), cudaMemcpyHostToDevice,
                                 s)) != cudaSuccess)
            return cfail("mask spans", e);
        // the host vectors must outlive the copies
        return (e = cudaStreamSynchronize(s)) == cudaSuccess ? 0 : cfail("sync", e);
    }

    // Copies, concealment and masks (no allocation, no sync: capturable).
    int enqueue_dropouts(cudaStream_t s)
    {
        cudaError_t e;
        const size_t flen = (size_t)g.field_width * g.field_height;
        for (const auto &c : cp.copies)
            if ((e = cudaMemcpy2DAsync(pool + (size_t)c.pool_field * pool_stride, pool_stride * sizeof(uint16_t),
                                       c.src, (size_t)c.src_stride * sizeof(uint16_t), flen * sizeof(uint16_t),
                                       (size_t)c.nfields, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                return cfail("concealment copy", e);
        if (!cp.frames.empty() &&
            chdg::dropout_apply(pool, pool_stride, g.field_width, d_idx, d_ops, d_idx + cp.frames.size(),
                                (int)cp.frames.size(), nullptr, g.field_height == 263, s) != 0)
            return cfail("concealment", cudaGetLastError());
        for (const auto &c : cp.clears)
            if ((e = cudaMemsetAsync(c.plane, 0, c.bytes, s)) != cudaSuccess) return cfail("mask clear", e);
        if (!cp.spans.empty()) {
            batch_mask_kernel<<<(unsigned)cp.spans.size(), 128, 0, s>>>(d_spans);
            if ((e = cudaGetLastError()) != cudaSuccess) return cfail("mask launch", e);
        }
        return 0;
    }

    void drop_graph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }

    static bool same(const std::vector<chdg_capture> &a, const chdg_capture *b, int n)
    {
        if ((int)a.size() != n) return false;
        for (int i = 0; i < n; i++)
            if (std::memcmp(&a[i], &b[i], sizeof(chdg_capture)) != 0) return false;
        return true;
    }

    int layout(const chdg_capture *caps, int n, const std::vector<int64_t> &pool_first, ModeLayout &m3,
               ModeLayout &m2)
    {
        // a capture's field i: in the concealment pool, or the caller's buffer
        auto field_ptr = [&](int ci, int64_t i) -> const uint16_t * {
            if (pool_first[(size_t)ci] >= 0) return pool + (size_t)(pool_first[(size_t)ci] + i) * pool_stride;
            return caps[ci].fields + i * caps[ci].field_stride;
        };
        const size_t fb = eng3.frame_bytes();
        for (int i = 0; i < n; i++) {
            const chdg_capture &k = caps[i];
            if (k.fields == nullptr || k.out == nullptr || k.nfields < 0 ||
                k.field_stride < (int64_t)g.field_width * g.field_height)
                return bfail("chdg_batch_decode: capture " + std::to_string(i) + " has bad arguments");
            if (k.kind != 7 && k.kind != 8)
                return bfail("chdg_batch_decode: capture kinds are 7 (Transform 2D) or 8 (Transform 3D)");
            if (!(k.threshold >= 0.0)) return bfail("chdg_batch_decode: negative threshold");
            (k.kind == 8 ? m3 : m2).caps.push_back(i);
        }
        auto frame_t2 = [](double t, float *dst) {
            const double t2 = t * t;
            dst[0] = (float)t2;
            dst[1] = (float)t2;
            dst[2] = (float)(t2 - (double)(float)t2);
        };
        // 3D: [gap][capture 0][gap][capture 1] ... [gap]
        int64_t fr = kGapFrames;
        for (int ci : m3.caps) {
            m3.first_frame.push_back(fr);
            fr += caps[ci].nfields / 2 + kGapFrames;
        }
        m3.frames = m3.caps.empty() ? 0 : fr;
        m3.fptr.assign((size_t)2 * m3.frames, nullptr);
        m3.t2.assign((size_t)3 * m3.frames, 0.f);
        m3.outs.assign((size_t)m3.frames, nullptr);
        for (size_t j = 0; j < m3.caps.size(); j++) {
            const chdg_capture &k = caps[m3.caps[j]];
            const int64_t a = m3.first_frame[j], nf = k.nfields / 2;
            // the capture's frames and the gap before it carry its threshold
            for (int64_t f = a - kGapFrames; f < a + nf; f++) frame_t2(k.threshold, &m3.t2[3 * f]);
            for (int64_t f = 0; f < nf; f++) m3.outs[a + f] = (char *)k.out + fb * (size_t)f;
            // an unpaired last field is outside every frame: black, as in the reference's window
            for (int64_t i = 0; i < 2 * nf; i++) m3.fptr[2 * a + i] = field_ptr(m3.caps[j], i);
        }
        int64_t fr2 = 0;
        for (int ci : m2.caps) {
            m2.first_frame.push_back(fr2);
            fr2 += caps[ci].nfields / 2;
        }
        m2.frames = fr2;
        m2.fptr.assign((size_t)2 * m2.frames, nullptr);
        m2.t2.assign((size_t)3 * m2.frames, 0.f);
        m2.outs.assign((size_t)m2.frames, nullptr);
        for (size_t j = 0; j < m2.caps.size(); j++) {
            const chdg_capture &k = caps[m2.caps[j]];
            const int64_t a = m2.first_frame[j], nf = k.nfields / 2;
            for (int64_t f = a; f < a + nf; f++) frame_t2(k.threshold, &m2.t2[3 * f]);
            for (int64_t f = 0; f < nf; f++) m2.outs[a + f] = (char *)k.out + fb * (size_t)f;
            for (int64_t i = 0; i < 2 * nf; i++) m2.fptr[2 * a + i] = field_ptr(m2.caps[j], i);
        }
        return 0;
    }

    // Upload one mode's tables (they depend only on the batch shape, so they
    // stay outside any graph).
    int upload(const ModeLayout &m, ModeTables &t, cudaStream_t s)
    {
        cudaError_t e;
        if (m.frames == 0) return 0;
        if ((size_t)m.frames > t.cap) {
            cudaFree(t.fptr);
            cudaFree(t.t2);
            cudaFree(t.outs);
            t.fptr = nullptr;
            t.t2 = nullptr;
            t.outs = nullptr;
            t.cap = 0;
            if ((e = cudaMalloc(&t.fptr, (size_t)m.frames * 2 * sizeof(void *))) != cudaSuccess ||
                (e = cudaMalloc(&t.t2, (size_t)m.frames * 3 * sizeof(float))) != cudaSuccess ||
                (e = cudaMalloc(&t.outs, (size_t)m.frames * sizeof(void *))) != cudaSuccess)
                return cfail("batch tables", e);
            t.cap = (size_t)m.frames;
        }
        if ((e = cudaMemcpyAsync(t.fptr, m.fptr.data(), m.fptr.size() * sizeof(void *), cudaMemcpyHostToDevice, s)) !=
                cudaSuccess ||
            (e = cudaMemcpyAsync(t.t2, m.t2.data(), m.t2.size() * sizeof(float), cudaMemcpyHostToDevice, s)) !=
                cudaSuccess ||
            (e = cudaMemcpyAsync(t.outs, m.outs.data(), m.outs.size() * sizeof(void *), cudaMemcpyHostToDevice, s)) !=
                cudaSuccess)
            return cfail("batch tables", e);
        return 0;
    }

    // Enqueue one mode's launches (no allocation, no sync: capturable into a
    // graph). Every field and frame has a table entry, so the engine's field
    // buffer and output arguments are placeholders.
    int enqueue(const chdg_capture *caps, const ModeLayout &m, chdg::Engine &eng, cudaStream_t s)
    {
        if (m.frames == 0) return 0;
        const long long flen = (long long)g.field_width * g.field_height;
        char dummy = 0;
        return eng.decode(caps[m.caps[0]].fields, flen, 0, (int)(2 * m.frames), 0, (int)m.frames, &dummy, s);
    }

    int run(const chdg_capture *caps, int n, cudaStream_t s, bool allow_graph)
    {
        // the legacy default stream cannot be captured: decode eagerly there
        if (s == nullptr) allow_graph = false;
        if (allow_graph && exec != nullptr && same(last, caps, n)) {
            const cudaError_t e = cudaGraphLaunch(exec, s);
            return e == cudaSuccess ? 0 : cfail("graph launch", e);
        }
        std::vector<int64_t> pool_first;
        if (const int rc = plan_dropouts(caps, n, pool_first); rc != 0) return rc;
        if (const int rc = upload_dropouts(s); rc != 0) return rc;
        ModeLayout m3, m2;
        if (const int rc = layout(caps, n, pool_first, m3, m2); rc != 0) return rc;
        if (const int rc = upload(m3, tab3, s); rc != 0) return rc;
        if (const int rc = upload(m2, tab2, s); rc != 0) return rc;
        cudaError_t e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cfail("sync", e);   // host tables may go
        eng3.set_frame_tables(tab3.fptr, tab3.t2, tab3.outs);
        eng2.set_frame_tables(tab2.fptr, tab2.t2, tab2.outs);
        const bool reshape = !same(last, caps, n);
        if (reshape) {
            drop_graph();
            last.assign(caps, caps + n);
            eager_runs = 0;
        }
        if (!allow_graph || eager_runs == 0) {
            // eager: sizes the engines' scratch before any capture
            eager_runs++;
            if (const int rc = enqueue_dropouts(s); rc != 0) return rc;
            if (const int rc = enqueue(caps, m3, eng3, s); rc != 0) return rc;
            return enqueue(caps, m2, eng2, s);
        }
        // capture this shape once, then replay
        if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cfail("begin capture", e);
        int rc = enqueue_dropouts(s);
        if (rc == 0) rc = enqueue(caps, m3, eng3, s);
        if (rc == 0) rc = enqueue(caps, m2, eng2, s);
        cudaGraph_t gph = nullptr;
        e = cudaStreamEndCapture(s, &gph);
        if (rc != 0) {
            if (gph) cudaGraphDestroy(gph);
            return rc;
        }
        if (e != cudaSuccess) return cfail("end capture", e);
        graph = gph;
        if ((e = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) {
            drop_graph();
            return cfail("graph instantiate", e);
        }
        if ((e = cudaGraphLaunch(exec, s)) != cudaSuccess) return cfail("graph launch", e);
        return 0;
    }
};

#pragma GCC visibility push(default)
extern "C" {

int chdg_batch_create(const chdg_geometry *g, const chdg_config *c, chdg_batch **out)
{
    if (g == nullptr || c == nullptr || out == nullptr) return bfail("chdg_batch_create: null argument");
    *out = nullptr;
    if (c->padding_multiple != 1) return bfail("chdg_batch_create: batches write unpadded frames (padding_multiple 1)");
    if (c->thresholds != nullptr) return bfail("chdg_batch_create: batches take one threshold per capture");
    auto b = std::make_unique<chdg_batch>();
    b->g = *g;
    b->c = *c;
    chdg_config c3 = *c, c2 = *c;
    c3.kind = 8;
    c2.kind = 7;
    if (const int rc = b->eng3.init(*g, c3); rc != 0) return rc;
    if (const int rc = b->eng2.init(*g, c2); rc != 0) return rc;
    *out = b.release();
    return 0;
}

void chdg_batch_free(chdg_batch *b) { delete b; }

int chdg_batch_decode(chdg_batch *b, const chdg_capture *caps, int32_t n, void *stream)
{
    if (b == nullptr || (n > 0 && caps == nullptr) || n < 0) return bfail("chdg_batch_decode: bad arguments");
    if (n == 0) return 0;
    return b->run(caps, n, (cudaStream_t)stream, true);
}

int chdg_batch_autotune(chdg_batch *b, const chdg_capture *caps, int32_t n, void *stream, chdg_batch_tuning *out)
{
    if (b == nullptr || caps == nullptr || n <= 0) return bfail("chdg_batch_autotune: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int chunks[] = {16, 24, 32, 48, 64};
    const int grids[] = {0, 3 * sms, 6 * sms};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = -1.f;
    int best_chunk = b->eng3.chunk_frames(), best_grid = b->eng3.max_blocks();
    // warm-up: sizes every buffer
    if (const int rc = b->run(caps, n, s, false); rc != 0) return rc;
    for (int ch : chunks)
        for (int gr : grids) {
            b->eng3.set_chunk_frames(ch);
            b->eng2.set_chunk_frames(ch);
            b->eng3.set_max_blocks(gr);
            cudaEventRecord(e0, s);
            if (const int rc = b->run(caps, n, s, false); rc != 0) return rc;
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (best < 0.f || ms < best) {
                best = ms;
                best_chunk = ch;
                best_grid = gr;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->eng3.set_chunk_frames(best_chunk);
    b->eng2.set_chunk_frames(best_chunk);
    b->eng3.set_max_blocks(best_grid);
    b->drop_graph();   // the next decode captures the tuned schedule
    b->last.clear();
    if (out != nullptr) {
        out->chunk_frames = best_chunk;
        out->max_blocks = best_grid;
        out->ms = best;
    }
    return 0;
}

}  // extern "C"
#pragma GCC visibility pop
