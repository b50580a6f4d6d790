// capture.h -- an opened ld-decode capture: the mmapped .tbc (uint16 fields)
// and its JSON sidecar (video parameters, per-field metadata, dropouts).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <chromadec/types.h>

namespace chdg {

enum System { SYS_PAL = 0, SYS_NTSC = 1, SYS_PAL_M = 2, SYS_SECAM = 3 };

// The VideoParameters fields this path reads (src/metadata/core.h:56-118).
struct VideoParams {
    int system = SYS_PAL;
    bool isSubcarrierLocked = false;
    bool isWidescreen = false;
    int fieldWidth = -1, fieldHeight = -1;
    double sampleRate = -1.0, fSC = -1.0;
    int activeVideoStart = -1, activeVideoEnd = -1;
    int colourBurstStart = -1, colourBurstEnd = -1;
    int white16bIre = -1, black16bIre = -1, blanking16bIre = -1;
    int firstActiveFrameLine = -1, lastActiveFrameLine = -1;
    int numberOfSequentialFields = -1;
};

struct Dropout {
    int32_t startx, endx, fieldLine;   // samples [startx, endx), 1-based field line
};

struct FieldMeta {
    bool isFirstField = false;
    bool pad = false;
    double bPSNR = 0.0;
    int32_t vbi[3] = {0, 0, 0};   // VBI lines 16-18 (Vbi::vbiData, src/metadata/core.h:46-53)
    std::vector<Dropout> dropouts;
};

// One field of a decode window (SourceField): where its samples come from.
struct WindowField {
    int source = 0;            // 1-based field number in the .tbc, 0 = black
    bool isFirstField = false;
    bool isPadding = false;
    int fieldNumber = 0;       // 1-based metadata field number (for dropouts)
};

class Capture {
public:
    Capture() = default;
    ~Capture();
    Capture(const Capture &) = delete;
    Capture &operator=(const Capture &) = delete;

    // Returns a chd_status_t value; sets the last-error detail on failure.
    int open(const char *path, const char *meta_or_null, const chd_video_params_t *override_or_null);

    const VideoParams &vp() const { return vp_; }
    const std::string &path() const { return path_; }
    int numMetadataFields() const { return (int)fields_.size(); }
    int numSourceFields() const { return nsource_; }
    bool isFirstFieldFirst() const { return firstFieldFirst_; }
    size_t fieldLen() const { return (size_t)vp_.fieldWidth * (size_t)vp_.fieldHeight; }

    // LdDecodeMetaData::getNumberOfFrames / getFieldNumber (src/metadata/core.cpp:1092-1190)
    int numFrames(bool firstFieldFirst) const;
    int fieldNumber(int frameNumber, int which, bool firstFieldFirst) const;
    const FieldMeta &field(int seq) const;        // 1-based; an empty field out of range
    const uint16_t *fieldData(int seq) const;     // 1-based field in the .tbc

    // The two fields of window frame `frameNumber` (1-based, may lie outside
    // the capture), with SourceField::loadFields' black-padding rules
    // (src/decoders/source_field.cpp:88-170).
    void windowFrame(int frameNumber, bool firstFieldFirst, WindowField out[2]) const;

private:
    std::string path_;
    VideoParams vp_;
    std::vector<FieldMeta> fields_;
    bool firstFieldFirst_ = true;
    int nsource_ = 0;
    int fd_ = -1;
    void *map_ = nullptr;
    size_t mapBytes_ = 0;
};

}  // namespace chdg
