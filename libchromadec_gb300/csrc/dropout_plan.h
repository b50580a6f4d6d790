// dropout_plan.h -- host-side planning of dropout concealment and dropout
// span mapping. The integer logic (span splitting, replacement-line search,
// statistics) runs on the host from metadata; the resulting ordered list of
// line operations is applied to the field samples on the GPU
// (dropout.cu), bit-exact with the reference's DropoutCorrector.
#pragma once

#include <cstdint>
#include <vector>

#include "capture.h"

namespace chdg {

// One concealment step on a frame's two fields (slot 0 / slot 1 of the
// window frame), applied in order.
struct DropOp {
    int32_t field;        // target slot
    int32_t mode;         // 1 = copy, 2 = low-frequency + high-frequency blend
    int32_t line;         // target field line, 0-based
    int32_t startx, endx; // samples [startx, endx)
    int32_t srcField, srcLine;   // replacement line (slot, 0-based line)
    int32_t chrField, chrLine;   // chroma replacement line (blend only)
    // Replacement lines from an extra capture: the field's index in the
    // plan's `extras` (on the device: in the batch's extra-field buffer),
    // -1 = the window slot srcField / chrField.
    int32_t srcExtra, chrExtra;
};

// A field of an extra capture that a plan reads replacement lines from.
struct ExtraField {
    const Capture *cap = nullptr;
    int32_t seq = 0;        // 1-based field number in its .tbc
    bool shifted = false;   // subcarrier-locked second field: samples 2.., then 2 black
    uint16_t black = 0;
};

struct FramePlan {
    std::vector<DropOp> ops;
    std::vector<ExtraField> extras;   // two per extra source (first, second)
    int32_t corrected = 0, failed = 0;
    int64_t totalDistance = 0;
};

// One extra capture's share of a frame's concealment (ExtraSourceFrame,
// src/dropout/dropout_corrector.h:47-55): its frame's fields as
// decodeSourceFrame reads them (first / second by its own pairing; the
// second's dropouts shifted when subcarrier-locked), its video parameters
// and its quality (average bPSNR of the two fields).
struct ExtraFrame {
    VideoParams vp;
    FieldMeta first, second;
    ExtraField firstField, secondField;
    double quality = 0.0;
};

// SourceField::secondFieldIsShifted (src/decoders/source_field.cpp:45-49):
// subcarrier-locked PAL and PAL-M captures store the second field of each
// window frame 2 samples late.
bool second_field_shifted(const VideoParams &vp);
// shiftSecondField's dropout move (source_field.cpp:59-65): 2 samples left,
// dropped when they end at or before sample 0.
FieldMeta shift_dropouts(const FieldMeta &f);

// DropoutCorrector::correctFrame (src/dropout/dropout_corrector.cpp:40-530),
// single source or with the extra captures that hold the frame. slot0/slot1
// are the frame's fields in window order.
FramePlan plan_frame(const VideoParams &vp, const FieldMeta &slot0, const FieldMeta &slot1, bool overcorrect,
                     bool intraField, const std::vector<ExtraFrame> &extras = {});

struct Span {
    int32_t y, x_start, x_end, origin;
};

// appendFieldSpans / collectSpans (src/abi/c_api_dropout_detect.cpp:92-174):
// both fields' dropouts in output framing, sorted by (y, x_start, x_end).
struct OutputFraming {
    int32_t activeVideoStart, activeWidth, width, height, firstActiveFrameLine, leftPad, topPad, fieldWidth;
};
std::vector<Span> frame_spans(const OutputFraming &g, const FieldMeta &slot0, bool slot0First,
                              const FieldMeta &slot1, bool slot1First, bool overcorrect);

}  // namespace chdg
