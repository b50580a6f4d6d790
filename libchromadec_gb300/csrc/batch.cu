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

#include "engine.h"
#include "error_state.h"

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
    // the shape of the last decode, and its graph
    std::vector<chdg_capture> last;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int eager_runs = 0;

    ~chdg_batch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
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

    int layout(const chdg_capture *caps, int n, ModeLayout &m3, ModeLayout &m2)
    {
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
            for (int64_t i = 0; i < 2 * nf; i++) m3.fptr[2 * a + i] = k.fields + i * k.field_stride;
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
            for (int64_t i = 0; i < 2 * nf; i++) m2.fptr[2 * a + i] = k.fields + i * k.field_stride;
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
        ModeLayout m3, m2;
        if (const int rc = layout(caps, n, m3, m2); rc != 0) return rc;
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
            if (const int rc = enqueue(caps, m3, eng3, s); rc != 0) return rc;
            return enqueue(caps, m2, eng2, s);
        }
        // capture this shape once, then replay
        if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cfail("begin capture", e);
        int rc = enqueue(caps, m3, eng3, s);
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
