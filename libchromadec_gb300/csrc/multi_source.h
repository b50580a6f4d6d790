// multi_source.h -- extra captures of the same disc for multi-source dropout
// concealment (chd_video_add_extra_source_*): the LaserDisc VBI codes that
// register them against the primary capture, and the alignment itself.
#pragma once

#include <cstdint>
#include <vector>

#include "capture.h"

namespace chdg {

// The VBI codes this path reads: CAV picture number and CLV time code
// (VbiDecoder::Vbi, src/metadata/vbi_decoder.h:59-67); -1 = absent.
struct VbiCodes {
    int32_t picNo = -1;
    int32_t clvHr = -1, clvMin = -1, clvSec = -1, clvPicNo = -1;
};

// VbiDecoder::decode for one field's lines 16-18 (IEC 60857-1986 10.1.3,
// 10.1.6, 10.1.10; src/metadata/vbi_decoder.cpp:131-232, 575-604).
VbiCodes decode_vbi_field(int32_t l16, int32_t l17, int32_t l18);
// VbiDecoder::decodeFrame: each code from the first field, else the second
// (vbi_decoder.cpp:49-80).
VbiCodes decode_vbi_frame(const int32_t first[3], const int32_t second[3]);
// LdDecodeMetaData::convertClvTimecodeToFrameNumber (src/metadata/core.cpp:1207-1238).
int32_t clv_frame_number(const VideoParams &vp, const VbiCodes &c);

// One capture of an alignment and the pairing order it is read with.
struct AlignedSource {
    const Capture *cap = nullptr;
    bool firstFieldFirst = true;
};

// MultiSourceAlignment (src/dropout/multi_source_alignment.cpp:37-201):
// source 0 is the primary; each source's disc-frame range comes from its
// CAV picture numbers or CLV time codes, and frame n of the primary maps to
// the frame of another source holding the same disc frame. Sources without
// VBI codes align positionally.
class SourceAlignment {
public:
    SourceAlignment() = default;
    // log: report each source's disc type and frame range at INFO, as the
    // reference does when a decode builds its alignment
    explicit SourceAlignment(std::vector<AlignedSource> sources, bool log = true);

    bool hasVbi(int s) const { return hasVbi_[(size_t)s]; }
    bool isCav(int s) const { return cav_[(size_t)s]; }
    int32_t minVbiFrame(int s) const { return minVbi_[(size_t)s]; }
    int32_t maxVbiFrame(int s) const { return maxVbi_[(size_t)s]; }
    // sourceFrameForPrimaryFrame: 1-based frame of source s, or -1.
    int32_t frameFor(int32_t primaryFrame, int s) const;

private:
    std::vector<AlignedSource> sources_;
    std::vector<bool> hasVbi_, cav_;
    std::vector<int32_t> minVbi_, maxVbi_;
};

// The extra captures a decoder conceals from, with their alignment to the
// primary (built once, on the first decode with concealment on).
struct MultiSource {
    std::vector<AlignedSource> extras;
    SourceAlignment alignment;   // over {primary, extras...}
};

}  // namespace chdg
