// ref_harness.cpp -- drives the reference's own Transform-PAL, PALcolour,
// OutputWriter and DropoutCorrector classes, compiled from the reference
// sources (see oracle/Makefile), on a raw field file. Test infrastructure: it
// produces the outputs that pin the C restatement in oracle/tpal_oracle.c.
//
// The per-frame flow mirrors the reference's decodeSourceFrame /
// decodeFrameLocked (src/abi/c_api_decoder.cpp:183-527): load a field window
// with black padding outside the capture (src/decoders/source_field.cpp:68-171),
// dropout-correct every non-padding window frame that has dropouts
// (c_api_decoder.cpp:300-321), run PalColour::decodeFrames, then
// OutputWriter::convert (yuv444p16) or convertToFloat (yuv444ps).
//
// Usage (key=value arguments):
//   mode=decode|chroma|dropout kind=2|3 fmt=p16|ps threshold=0.4
//   thresholds=<file> in=<fields.u16> nfields=N first=F count=C out=<file>
//   dropouts=<file> overcorrect=0|1 intra=0|1
//   gain=<chroma gain> phase=<degrees> clamp=0..3 padding=<multiple>
//   avs=<first active sample> ave=<one past the last> fafl=<first active
//   frame line> lafl=<last active frame line>
//   kind=1 (PALcolour 2D filter alone) fmt=rgb48|rgbs|gray16|grays
//   ynr=<luma_nr_level> sff=1 (window slot 0 holds second fields: the
//   reversed pairing) sclocked=1 (subcarrier-locked: slot-1 fields shifted)
//   cdp=classic|modern bsp=classic|modern|scientific
//   extra1=<fields>:<nfields>:<dropout file or ->:<frame offset> (up to
//   extra8): extra captures for multi-source concealment; window frame f
//   takes frame f + offset of the extra, positionally as the reference's
//   MultiSourceAlignment does without VBI codes
//   (src/dropout/multi_source_alignment.cpp:54-71), skipped when the extra
//   does not hold it (src/abi/c_api_decoder.cpp:252-262)
//   bpsnr=<file>: lines "source field bPSNR" (source 0 = primary)
//   std=pal|palm: the video standard (default pal)
// The field file holds N fields of 1135x313 (PAL-M 909x263) uint16, first
// field first.
// The dropout file holds lines "field_index startx endx fieldLine".

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "common/color_conversion.h"
#include "decoders/palcolour/palcolour.h"
#include "decoders/palcolour/transform_pal_2d.h"
#include "decoders/palcolour/transform_pal_3d.h"
#include "decoders/source_field.h"
#include "dropout/dropout_corrector.h"
#include "output/component_frame.h"
#include "output/output_writer.h"

using chd::metadata::LdDecodeMetaData;

namespace {

// Line-locked 4fsc PAL geometry: the reference's own preset values
// (src/format/video_standards.cpp:58-70,116-207 and src/metadata/core.cpp:40-50).
LdDecodeMetaData::VideoParameters palParams()
{
    LdDecodeMetaData::VideoParameters vp;
    vp.system = chd::metadata::PAL;
    vp.isSubcarrierLocked = false;
    vp.fieldWidth = 1135;
    vp.fieldHeight = 313;
    vp.sampleRate = 4.0 * 625.0 * 25.0 * (1135.0 / 4.0 + 1.0 / 625.0);
    vp.fSC = 283.75 * 15625.0 + 25.0;
    vp.colourBurstStart = 98;
    vp.colourBurstEnd = 138;
    vp.activeVideoStart = 177;
    vp.activeVideoEnd = 1125;
    vp.black16bIre = 256 * 64;
    vp.white16bIre = 844 * 64;
    vp.blanking16bIre = 256 * 64;
    vp.firstActiveFrameLine = 44;
    vp.lastActiveFrameLine = 619;
    vp.pictureStart = vp.activeVideoStart;
    vp.pictureEnd = vp.activeVideoEnd;
    vp.tileReadStart = vp.activeVideoStart;
    vp.tileReadEnd = vp.activeVideoEnd;
    vp.isValid = true;
    return vp;
}

// PAL-M: the reference's PAL_M preset (src/format/video_standards.cpp:28-52,
// 85-100, 116-207, sync-start rows) and its active frame lines
// (src/metadata/core.cpp:52-70): 909 x 263 fields at 4 fSC, ST 244 levels.
LdDecodeMetaData::VideoParameters palMParams()
{
    LdDecodeMetaData::VideoParameters vp = palParams();
    vp.system = chd::metadata::PAL_M;
    vp.fieldWidth = 909;
    vp.fieldHeight = 263;
    vp.sampleRate = 4.0 * 525.0 * (30000.0 / 1001.0) * (909.0 / 4.0);
    vp.fSC = 5.0e6 * (63.0 / 88.0) * (909.0 / 910.0);
    vp.colourBurstStart = 75;
    vp.colourBurstEnd = 95;
    vp.activeVideoStart = 124;
    vp.activeVideoEnd = 892;
    vp.black16bIre = 282 * 64;
    vp.white16bIre = 800 * 64;
    vp.blanking16bIre = 240 * 64;
    vp.firstActiveFrameLine = 39;
    vp.lastActiveFrameLine = 524;
    vp.pictureStart = vp.activeVideoStart;
    vp.pictureEnd = vp.activeVideoEnd;
    vp.tileReadStart = vp.activeVideoStart;
    vp.tileReadEnd = vp.activeVideoEnd;
    return vp;
}

std::map<std::string, std::string> parseArgs(int argc, char **argv)
{
    std::map<std::string, std::string> m;
    for (int i = 1; i < argc; i++) {
        const char *eq = std::strchr(argv[i], '=');
        if (!eq) continue;
        m[std::string(argv[i], eq - argv[i])] = std::string(eq + 1);
    }
    return m;
}

struct Capture {
    std::vector<uint16_t> samples;
    int nfields = 0;
    size_t fieldLen = 0;
    std::vector<chd::metadata::DropOuts> dropouts;  // per field
    std::vector<double> bpsnr;                       // per field
    int frameOffset = 0;                             // extras: window frame f is this capture's f + offset
};

bool readFields(const std::string &path, Capture &cap)
{
    cap.samples.resize(cap.fieldLen * cap.nfields);
    FILE *fp = std::fopen(path.c_str(), "rb");
    if (!fp) return false;
    const bool ok = std::fread(cap.samples.data(), 2, cap.samples.size(), fp) == cap.samples.size();
    std::fclose(fp);
    return ok;
}

void readDropouts(const std::string &path, Capture &cap)
{
    cap.dropouts.assign(cap.nfields, chd::metadata::DropOuts());
    cap.bpsnr.assign(cap.nfields, 0.0);
    if (path.empty() || path == "-") return;
    std::ifstream in(path);
    int fi, sx, ex, fl;
    while (in >> fi >> sx >> ex >> fl) {
        if (fi >= 0 && fi < cap.nfields) cap.dropouts[fi].append(sx, ex, fl);
    }
}

// Field window for frames [firstFrame - lookBehind, firstFrame + 1 + lookAhead),
// black padding outside the capture (source_field.cpp:88-170).
void loadWindow(const Capture &cap, const LdDecodeMetaData::VideoParameters &vp, int frame, int lookBehind,
                int lookAhead, bool slot0IsSecond, std::vector<chd::decoders::SourceField> &fields,
                int &startIndex, int &endIndex)
{
    startIndex = 2 * lookBehind;
    endIndex = startIndex + 2;
    fields.assign(endIndex + 2 * lookAhead, chd::decoders::SourceField());
    const int numFrames = cap.nfields / 2;
    for (size_t i = 0; i < fields.size(); i += 2) {
        const int f = frame - lookBehind + static_cast<int>(i / 2);
        const bool pad = f < 0 || f >= numFrames;
        for (int j = 0; j < 2; j++) {
            auto &sf = fields[i + j];
            sf.field.isFirstField = slot0IsSecond ? (j == 1) : (j == 0);
            sf.isPadding = pad;
            const int srcField = pad ? j : 2 * f + j;
            sf.fieldNumber = srcField + 1;
            sf.field.dropOuts = cap.dropouts[srcField];
            sf.field.vitsMetrics.bPSNR = cap.bpsnr[srcField];
            if (pad) {
                sf.data.assign(cap.fieldLen, static_cast<uint16_t>(vp.black16bIre));
            } else {
                sf.data.assign(cap.samples.begin() + cap.fieldLen * srcField,
                               cap.samples.begin() + cap.fieldLen * (srcField + 1));
                if (j == 1 && chd::decoders::SourceField::secondFieldIsShifted(vp))
                    chd::decoders::SourceField::shiftSecondField(sf.data, sf.field.dropOuts,
                                                                 static_cast<uint16_t>(vp.black16bIre));
            }
        }
    }
}

}  // namespace

int main(int argc, char **argv)
{
    auto a = parseArgs(argc, argv);
    const std::string mode = a.count("mode") ? a["mode"] : "decode";
    const int kind = a.count("kind") ? std::atoi(a["kind"].c_str()) : 3;
    const std::string fmt = a.count("fmt") ? a["fmt"] : "p16";
    const double threshold = a.count("threshold") ? std::atof(a["threshold"].c_str()) : 0.4;
    const int first = a.count("first") ? std::atoi(a["first"].c_str()) : 0;
    const int count = a.count("count") ? std::atoi(a["count"].c_str()) : 1;
    const bool overcorrect = a.count("overcorrect") && a["overcorrect"] == "1";
    const bool intra = a.count("intra") && a["intra"] == "1";

    auto vp = (a.count("std") && a["std"] == "palm") ? palMParams() : palParams();
    if (a.count("avs")) vp.activeVideoStart = vp.pictureStart = vp.tileReadStart = std::atoi(a["avs"].c_str());
    if (a.count("ave")) vp.activeVideoEnd = vp.pictureEnd = vp.tileReadEnd = std::atoi(a["ave"].c_str());
    if (a.count("fafl")) vp.firstActiveFrameLine = std::atoi(a["fafl"].c_str());
    if (a.count("lafl")) vp.lastActiveFrameLine = std::atoi(a["lafl"].c_str());
    if (a.count("sclocked") && a["sclocked"] == "1") vp.isSubcarrierLocked = true;
    const bool slot0IsSecond = a.count("sff") && a["sff"] == "1";
    Capture cap;
    cap.nfields = std::atoi(a["nfields"].c_str());
    cap.fieldLen = static_cast<size_t>(vp.fieldWidth) * vp.fieldHeight;
    if (!readFields(a["in"], cap)) {
        std::fprintf(stderr, "ref_harness: cannot read %s\n", a["in"].c_str());
        return 2;
    }
    const bool correcting = a.count("dropouts") != 0;
    readDropouts(correcting ? a["dropouts"] : std::string(), cap);
    std::vector<Capture> extras;
    for (int e = 1; e <= 8; e++) {
        const std::string key = "extra" + std::to_string(e);
        if (!a.count(key)) break;
        // <fields>:<nfields>:<dropouts>:<offset>
        std::vector<std::string> parts;
        std::string cur;
        for (char ch : a[key]) {
            if (ch == ':') {
                parts.push_back(cur);
                cur.clear();
            } else {
                cur += ch;
            }
        }
        parts.push_back(cur);
        if (parts.size() != 4) return 2;
        Capture x;
        x.nfields = std::atoi(parts[1].c_str());
        x.fieldLen = cap.fieldLen;
        if (!readFields(parts[0], x)) {
            std::fprintf(stderr, "ref_harness: cannot read %s\n", parts[0].c_str());
            return 2;
        }
        readDropouts(parts[2], x);
        x.frameOffset = std::atoi(parts[3].c_str());
        extras.push_back(std::move(x));
    }
    if (a.count("bpsnr")) {
        std::ifstream in(a["bpsnr"]);
        int src, fi;
        double v;
        while (in >> src >> fi >> v) {
            Capture &c = (src == 0) ? cap : extras.at(src - 1);
            if (fi >= 0 && fi < c.nfields) c.bpsnr[fi] = v;
        }
    }

    chd::decoders::palcolour::PalColour::Configuration cfg;
    cfg.separation = (kind == 1)   ? chd::decoders::palcolour::PalColour::palColourFilter
                     : (kind == 2) ? chd::decoders::palcolour::PalColour::transform2DFilter
                                   : chd::decoders::palcolour::PalColour::transform3DFilter;
    if (a.count("ynr")) cfg.yNRLevel = std::atof(a["ynr"].c_str());
    chd::color::ColorDifferencePrecision cdp = chd::color::ColorDifferencePrecision::Modern;
    chd::color::BroadcastScalingPrecision bsp = chd::color::BroadcastScalingPrecision::Scientific;
    if (a.count("cdp")) cdp = *chd::color::parseColorDifferencePrecision(a["cdp"]);
    if (a.count("bsp")) bsp = *chd::color::parseBroadcastScalingPrecision(a["bsp"]);
    cfg.colorConversion = chd::color::resolveColorConversion(cdp, bsp);
    cfg.transformThreshold = threshold;
    if (a.count("gain")) cfg.chromaGain = std::atof(a["gain"].c_str());
    if (a.count("phase")) cfg.chromaPhase = std::atof(a["phase"].c_str());
    if (a.count("thresholds")) {
        std::ifstream in(a["thresholds"]);
        double v;
        while (in >> v) cfg.transformThresholds.push_back(v);
    }
    const int lookBehind = cfg.getLookBehind();
    const int lookAhead = cfg.getLookAhead();

    FILE *out = std::fopen(a["out"].c_str(), "wb");
    if (!out) return 3;

    chd::decoders::palcolour::PalColour pal;
    pal.updateConfiguration(vp, cfg);

    std::unique_ptr<chd::decoders::palcolour::TransformPal> tp;
    if (mode == "chroma") {
        if (kind == 2) tp = std::make_unique<chd::decoders::palcolour::TransformPal2D>();
        else tp = std::make_unique<chd::decoders::palcolour::TransformPal3D>();
        tp->updateConfiguration(vp, cfg.transformThreshold, cfg.transformThresholds, cfg.colorConversion);
    }

    chd::output::OutputWriter writer;
    chd::output::OutputWriter::Configuration ocfg;
    ocfg.paddingAmount = a.count("padding") ? std::atoi(a["padding"].c_str()) : 1;
    ocfg.pixelFormat = (fmt == "rgb48") ? chd::output::OutputWriter::RGB48
                       : (fmt == "gray16") ? chd::output::OutputWriter::GRAY16
                                           : chd::output::OutputWriter::YUV444P16;
    ocfg.colorDifferencePrecision = cdp;
    ocfg.broadcastScalingPrecision = bsp;
    if (a.count("clamp"))
        ocfg.clampMode = static_cast<chd::output::OutputWriter::ClampMode>(std::atoi(a["clamp"].c_str()));
    writer.updateConfiguration(vp, ocfg);

    long totalCorrected = 0, totalFailed = 0;
    long long totalDistance = 0;
    for (int frame = first; frame < first + count; frame++) {
        std::vector<chd::decoders::SourceField> fields;
        int startIndex = 0, endIndex = 0;
        const int lb = (mode == "dropout") ? 0 : lookBehind;
        const int la = (mode == "dropout") ? 0 : lookAhead;
        loadWindow(cap, vp, frame, lb, la, slot0IsSecond, fields, startIndex, endIndex);

        if (correcting) {
            for (size_t i = 0; i + 1 < fields.size(); i += 2) {
                if (fields[i].isPadding) continue;
                if (fields[i].field.dropOuts.empty() && fields[i + 1].field.dropOuts.empty()) continue;
                chd::dropout::DropoutCorrector corrector(vp);
                chd::dropout::DropoutCorrectionStats stats;
                // The extras that hold this window frame, read the way
                // decodeSourceFrame does (src/abi/c_api_decoder.cpp:245-282):
                // slot 0 as "first", slot 1 (shifted when subcarrier-locked)
                // as "second", quality the fields' average bPSNR.
                const int f = frame - lb + static_cast<int>(i / 2);
                std::vector<chd::dropout::ExtraSourceFrame> ex;
                for (const Capture &x : extras) {
                    const int k = f + x.frameOffset;
                    if (k < 0 || k >= x.nfields / 2) continue;
                    chd::dropout::ExtraSourceFrame esf;
                    esf.firstFieldData.assign(x.samples.begin() + x.fieldLen * (2 * k),
                                              x.samples.begin() + x.fieldLen * (2 * k + 1));
                    esf.secondFieldData.assign(x.samples.begin() + x.fieldLen * (2 * k + 1),
                                               x.samples.begin() + x.fieldLen * (2 * k + 2));
                    esf.firstFieldMeta.dropOuts = x.dropouts[2 * k];
                    esf.secondFieldMeta.dropOuts = x.dropouts[2 * k + 1];
                    esf.firstFieldMeta.vitsMetrics.bPSNR = x.bpsnr[2 * k];
                    esf.secondFieldMeta.vitsMetrics.bPSNR = x.bpsnr[2 * k + 1];
                    esf.videoParams = vp;
                    if (chd::decoders::SourceField::secondFieldIsShifted(esf.videoParams))
                        chd::decoders::SourceField::shiftSecondField(esf.secondFieldData, esf.secondFieldMeta.dropOuts,
                                                                     static_cast<uint16_t>(vp.black16bIre));
                    esf.quality = (esf.firstFieldMeta.vitsMetrics.bPSNR + esf.secondFieldMeta.vitsMetrics.bPSNR) / 2.0;
                    ex.push_back(std::move(esf));
                }
                // correctFrame orders the pair by isFirstField itself
                if (ex.empty())
                    corrector.correctFrame(fields[i], fields[i + 1], overcorrect, intra, &stats);
                else
                    corrector.correctFrame(fields[i], fields[i + 1], ex, overcorrect, intra, &stats);
                if (static_cast<int>(i) == startIndex) {
                    totalCorrected += stats.corrected;
                    totalFailed += stats.failed;
                    totalDistance += stats.totalDistance;
                }
            }
        }

        if (mode == "dropout") {
            std::fwrite(fields[startIndex].data.data(), 2, cap.fieldLen, out);
            std::fwrite(fields[startIndex + 1].data.data(), 2, cap.fieldLen, out);
            continue;
        }
        if (mode == "chroma") {
            std::vector<const double *> chroma(endIndex - startIndex);
            tp->filterFields(fields, startIndex, endIndex, chroma);
            for (const double *c : chroma) std::fwrite(c, sizeof(double), cap.fieldLen, out);
            continue;
        }

        std::vector<chd::output::ComponentFrame> frames(1);
        pal.decodeFrames(fields, startIndex, endIndex, frames);
        if (fmt == "ps" || fmt == "grays") {
            std::vector<float> planes[3];
            writer.convertToFloat(frames[0], planes, fmt == "ps");
            for (int p = 0; p < 3; p++) std::fwrite(planes[p].data(), sizeof(float), planes[p].size(), out);
        } else if (fmt == "rgbs") {
            std::vector<float> planes[3];
            writer.convertToFloatRGB(frames[0], planes);
            for (int p = 0; p < 3; p++) std::fwrite(planes[p].data(), sizeof(float), planes[p].size(), out);
        } else {
            chd::output::OutputFrame of;
            writer.convert(frames[0], of);
            std::fwrite(of.data(), 2, of.size(), out);
        }
    }
    std::fclose(out);
    std::printf("{\"corrected\": %ld, \"failed\": %ld, \"total_distance\": %lld}\n", totalCorrected, totalFailed,
                totalDistance);
    return 0;
}
