// multi_source.cpp -- see multi_source.h. Each function cites the reference
// code it follows.
#include "multi_source.h"

#include <string>

#include "log_sink.h"

namespace chdg {

namespace {

// VbiDecoder::decodeBCD (src/metadata/vbi_decoder.cpp:650-668): writes the
// value only when every nibble is a decimal digit.
bool bcd(uint32_t v, int32_t &out)
{
    int32_t value = 0;
    uint32_t place = 1;
    while (v != 0) {
        const uint32_t digit = v & 0xF;
        if (digit > 9) return false;
        value += (int32_t)(digit * place);
        place *= 10;
        v >>= 4;
    }
    out = value;
    return true;
}

}  // namespace

VbiCodes decode_vbi_field(int32_t l16, int32_t l17, int32_t l18)
{
    VbiCodes v;
    if (l16 == -1 && l17 == -1 && l18 == -1) return v;
    // 10.1.3 CAV picture number on line 17 or 18 (first digit 0-7)
    for (const int32_t l : {l17, l18})
        if (((uint32_t)l & 0xF00000u) == 0xF00000u) bcd((uint32_t)l & 0x07FFFFu, v.picNo);
    // 10.1.6 CLV programme time code: hour and minutes must both be valid
    for (const int32_t l : {l17, l18}) {
        if (((uint32_t)l & 0xF0FF00u) == 0xF0DD00u) {
            int32_t hour;
            if (bcd(((uint32_t)l & 0x0F0000u) >> 16, hour) && bcd((uint32_t)l & 0x0000FFu, v.clvMin)) v.clvHr = hour;
        }
    }
    // 10.1.10 CLV picture number on line 16: seconds' first digit is A-F
    if (((uint32_t)l16 & 0xF0F000u) == 0x80E000u) {
        const uint32_t x1 = ((uint32_t)l16 & 0x0F0000u) >> 16;
        int32_t sec;
        if (x1 >= 0xA && bcd(((uint32_t)l16 & 0x000F00u) >> 8, sec) && bcd((uint32_t)l16 & 0x0000FFu, v.clvPicNo)) {
            v.clvSec = (10 * (int32_t)(x1 - 0xA)) + sec;
            v.picNo = -1;   // a CLV picture number invalidates the CAV one
        }
    }
    return v;
}

VbiCodes decode_vbi_frame(const int32_t first[3], const int32_t second[3])
{
    const VbiCodes a = decode_vbi_field(first[0], first[1], first[2]);
    const VbiCodes b = decode_vbi_field(second[0], second[1], second[2]);
    VbiCodes v;
    v.picNo = (a.picNo != -1) ? a.picNo : b.picNo;
    v.clvHr = (a.clvHr != -1) ? a.clvHr : b.clvHr;
    v.clvMin = (a.clvMin != -1) ? a.clvMin : b.clvMin;
    v.clvSec = (a.clvSec != -1) ? a.clvSec : b.clvSec;
    v.clvPicNo = (a.clvPicNo != -1) ? a.clvPicNo : b.clvPicNo;
    return v;
}

int32_t clv_frame_number(const VideoParams &vp, const VbiCodes &c)
{
    if (c.clvHr == -1 || c.clvMin == -1 || c.clvSec == -1 || c.clvPicNo == -1) return -1;
    const int32_t fps = (vp.system == SYS_PAL) ? 25 : 30;
    return c.clvHr * 3600 * fps + c.clvMin * 60 * fps + c.clvSec * fps + c.clvPicNo;
}

// setMinAndMaxVbiFrames (multi_source_alignment.cpp:73-162)
SourceAlignment::SourceAlignment(std::vector<AlignedSource> sources, bool log) : sources_(std::move(sources))
{
    const size_t n = sources_.size();
    hasVbi_.assign(n, false);
    cav_.assign(n, false);
    minVbi_.assign(n, 0);
    maxVbi_.assign(n, 0);
    for (size_t s = 0; s < n; s++) {
        const Capture &cap = *sources_[s].cap;
        const bool ffF = sources_[s].firstFieldFirst;
        int32_t cavCount = 0, clvCount = 0;
        int32_t cavMin = 1000000, cavMax = 0, clvMin = 1000000, clvMax = 0;
        const int frames = cap.numFrames(ffF);
        for (int f = 1; f <= frames; f++) {
            // getFieldVbi of an out-of-range field number is the empty field's {0, 0, 0}
            const FieldMeta &a = cap.field(cap.fieldNumber(f, 1, ffF));
            const FieldMeta &b = cap.field(cap.fieldNumber(f, 2, ffF));
            const VbiCodes v = decode_vbi_frame(a.vbi, b.vbi);
            if (v.picNo > 0) {
                cavCount++;
                if (v.picNo < cavMin) cavMin = v.picNo;
                if (v.picNo > cavMax) cavMax = v.picNo;
            }
            if (v.clvHr != -1 && v.clvMin != -1 && v.clvSec != -1 && v.clvPicNo != -1) {
                clvCount++;
                const int32_t fn = clv_frame_number(cap.vp(), v);
                if (fn < clvMin) clvMin = fn;
                if (fn > clvMax) clvMax = fn;
            }
        }
        if (cavCount == 0 && clvCount == 0) continue;   // no VBI: aligned positionally
        hasVbi_[s] = true;
        cav_[s] = cavCount > clvCount;
        minVbi_[s] = cav_[s] ? cavMin : clvMin;
        maxVbi_[s] = cav_[s] ? cavMax : clvMax;
        if (log) {
            const std::string msg = "Source #" + std::to_string(s);
            log_emit(CHD_LOG_INFO, 0,
                     (msg + (cav_[s] ? " has a disc type of CAV (uses VBI frame numbers)"
                                     : " has a disc type of CLV (uses VBI time codes)"))
                         .c_str());
            log_emit(CHD_LOG_INFO, 0,
                     (msg + " has a VBI frame number range of " + std::to_string(minVbi_[s]) + " to " +
                      std::to_string(maxVbi_[s]))
                         .c_str());
        }
    }
}

// sourceFrameForPrimaryFrame and the sequential <-> VBI conversions
// (multi_source_alignment.cpp:54-71, 164-177)
int32_t SourceAlignment::frameFor(int32_t primaryFrame, int s) const
{
    if (s == 0) return primaryFrame;
    if (!hasVbi_[0] || !hasVbi_[(size_t)s]) return primaryFrame;
    const int32_t vbiFrame = (minVbi_[0] - 1) + primaryFrame;
    if (vbiFrame >= minVbi_[(size_t)s] && vbiFrame <= maxVbi_[(size_t)s]) return vbiFrame - minVbi_[(size_t)s] + 1;
    return -1;
}

}  // namespace chdg
