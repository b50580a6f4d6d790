// dropout_plan.cpp -- integer planning of dropout concealment; see
// dropout_plan.h. Each function cites the reference code it follows.
#include "dropout_plan.h"

#include <algorithm>
#include <cstdlib>

namespace chdg {

namespace {

enum Loc { VISIBLE = 0, BURST = 1, UNKNOWN = 2 };

struct DLoc {
    int32_t fieldLine, startx, endx, location;
};

// populateDropoutsVector, dropout_corrector.cpp:160-193
std::vector<DLoc> populate(const VideoParams &vp, const FieldMeta &f, bool overCorrect)
{
    std::vector<DLoc> out;
    for (const Dropout &d : f.dropouts) {
        DLoc l{d.fieldLine, d.startx, d.endx, UNKNOWN};
        if (l.fieldLine < 1 || l.fieldLine > vp.fieldHeight) continue;
        if (overCorrect) {
            const int32_t dots = 24;
            l.startx = (l.startx > dots) ? l.startx - dots : 0;
            l.endx = (l.endx < vp.fieldWidth - dots) ? l.endx + dots : vp.fieldWidth;
        }
        out.push_back(l);
    }
    return out;
}

// setDropOutLocations, dropout_corrector.cpp:196-245
void set_locations(const VideoParams &vp, std::vector<DLoc> &d)
{
    int32_t splits;
    do {
        const size_t n = d.size();
        splits = 0;
        for (size_t i = 0; i < n; i++) {
            if (d[i].startx <= vp.colourBurstEnd) {
                d[i].location = BURST;
                if (d[i].endx > vp.colourBurstEnd) {
                    d.push_back({d[i].fieldLine, vp.colourBurstEnd + 1, d[i].endx, BURST});
                    d[i].endx = vp.colourBurstEnd;
                    splits++;
                }
            } else if (d[i].startx > vp.colourBurstEnd && d[i].startx <= vp.activeVideoEnd) {
                d[i].location = VISIBLE;
                if (d[i].endx > vp.activeVideoEnd) {
                    d[i].endx = vp.activeVideoEnd;
                    splits++;
                }
            }
        }
    } while (splits != 0);
}

struct Rep {
    bool sameField = true;
    int32_t fieldLine = -1;
    double quality = -1.0;
    int32_t distance = 0;
};

// findPotentialReplacementLine, dropout_corrector.cpp:417-466
void find_potential(const VideoParams &vp, const std::vector<DLoc> &target, size_t ti,
                    const std::vector<DLoc> &source, bool sameField, int32_t offset, int32_t step, double quality,
                    std::vector<Rep> &cands)
{
    const int32_t firstF = (vp.firstActiveFrameLine + 1) / 2;   // firstActiveFieldLine()
    const int32_t lastF = vp.lastActiveFrameLine / 2;           // lastActiveFieldLine()
    int32_t line = target[ti].fieldLine + offset;
    if ((line - 1) < firstF || (line - 1) > lastF) return;
    while ((line - 1) >= firstF && line <= lastF) {
        bool overlap = false;
        for (const DLoc &s : source) {
            if (s.fieldLine == line && (target[ti].endx - s.startx) >= 0 && (s.endx - target[ti].startx) >= 0) {
                line += step;
                overlap = true;
                break;
            }
        }
        if (!overlap) {
            Rep r;
            r.sameField = sameField;
            r.fieldLine = line;
            r.quality = quality;
            cands.push_back(r);
            return;
        }
    }
}

// findReplacementLine, dropout_corrector.cpp:248-414 (single source)
Rep find_replacement(const VideoParams &vp, const std::vector<DLoc> &thisD, const std::vector<DLoc> &otherD,
                     size_t idx, bool thisFieldIsFirst, bool matchChromaPhase, bool isColourBurst, bool intraField,
                     double quality)
{
    int32_t step, otherOffset;
    if (!matchChromaPhase) {
        step = 1;
        otherOffset = -1;
    } else if (vp.system == SYS_PAL || vp.system == SYS_PAL_M) {
        step = 4;
        otherOffset = thisFieldIsFirst ? -3 : -1;
    } else if (vp.system == SYS_SECAM) {
        step = 2;
        otherOffset = -1;
    } else {
        step = 2;
        otherOffset = -1;
    }
    std::vector<Rep> cands;
    find_potential(vp, thisD, idx, thisD, true, 0, -step, quality, cands);
    find_potential(vp, thisD, idx, thisD, true, step, step, quality, cands);
    if (!isColourBurst && !intraField) {
        find_potential(vp, thisD, idx, otherD, false, otherOffset, -step, quality, cands);
        find_potential(vp, thisD, idx, otherD, false, otherOffset + step, step, quality, cands);
    }
    Rep rep;
    if (!cands.empty()) {
        rep.distance = 1000000;
        rep.quality = -1;
        for (const Rep &c : cands) {
            const int32_t dropLine = (2 * thisD[idx].fieldLine) + (thisFieldIsFirst ? 0 : 1);
            const int32_t srcLine = (2 * c.fieldLine) + (c.sameField ? (thisFieldIsFirst ? 0 : 1) : (thisFieldIsFirst ? 1 : 0));
            const int32_t distance = std::abs(dropLine - srcLine);
            if (distance < rep.distance) {
                rep = c;
                rep.distance = distance;
            } else if (distance == rep.distance && c.quality > rep.quality) {
                rep = c;
                rep.distance = distance;
            }
        }
    }
    return rep;
}

// correctField + correctDropOut's choice of operation
// (dropout_corrector.cpp:117-157, 469-530)
void plan_field(const VideoParams &vp, const std::vector<DLoc> &thisD, const std::vector<DLoc> &otherD, int thisSlot,
                int otherSlot, bool thisFieldIsFirst, bool intraField, double quality, FramePlan &plan)
{
    for (size_t i = 0; i < thisD.size(); i++) {
        Rep rep, crep;
        if (thisD[i].location == BURST)
            rep = find_replacement(vp, thisD, otherD, i, thisFieldIsFirst, true, true, intraField, quality);
        if (thisD[i].location == VISIBLE) {
            rep = find_replacement(vp, thisD, otherD, i, thisFieldIsFirst, false, false, intraField, quality);
            crep = find_replacement(vp, thisD, otherD, i, thisFieldIsFirst, true, false, intraField, quality);
        }
        if (rep.fieldLine == -1) {
            plan.failed++;
            continue;
        }
        plan.corrected++;
        plan.totalDistance += rep.distance;
        DropOp op{};
        op.field = thisSlot;
        op.line = thisD[i].fieldLine - 1;
        op.startx = thisD[i].startx;
        op.endx = thisD[i].endx;
        op.srcField = rep.sameField ? thisSlot : otherSlot;
        op.srcLine = rep.fieldLine - 1;
        if (crep.fieldLine == -1 || (thisD[i].fieldLine == rep.fieldLine && thisD[i].fieldLine == crep.fieldLine)) {
            op.mode = 1;
        } else {
            op.mode = 2;
            op.chrField = crep.sameField ? thisSlot : otherSlot;
            op.chrLine = crep.fieldLine - 1;
        }
        plan.ops.push_back(op);
    }
}

}  // namespace

bool second_field_shifted(const VideoParams &vp)
{
    return (vp.system == SYS_PAL || vp.system == SYS_PAL_M) && vp.isSubcarrierLocked;
}

FieldMeta shift_dropouts(const FieldMeta &f)
{
    FieldMeta out = f;
    out.dropouts.clear();
    for (const Dropout &d : f.dropouts) {
        const int32_t endx = d.endx - 2;
        if (endx > 0) out.dropouts.push_back({std::max(d.startx - 2, 0), endx, d.fieldLine});
    }
    return out;
}

FramePlan plan_frame(const VideoParams &vp, const FieldMeta &slot0, const FieldMeta &slot1, bool overcorrect,
                     bool intraField)
{
    FramePlan plan;
    // broadcast order (dropout_corrector.cpp:56-57)
    const bool s0first = slot0.isFirstField;
    const FieldMeta &bf = s0first ? slot0 : slot1;
    const FieldMeta &bs = s0first ? slot1 : slot0;
    const int bfSlot = s0first ? 0 : 1, bsSlot = s0first ? 1 : 0;
    if (bf.dropouts.empty() && bs.dropouts.empty()) return plan;
    const double quality = (bf.bPSNR + bs.bPSNR) / 2.0;
    std::vector<DLoc> fd, sd;
    if (!bf.dropouts.empty()) {
        fd = populate(vp, bf, overcorrect);
        set_locations(vp, fd);
    }
    if (!bs.dropouts.empty()) {
        sd = populate(vp, bs, overcorrect);
        set_locations(vp, sd);
    }
    plan_field(vp, fd, sd, bfSlot, bsSlot, true, intraField, quality, plan);
    plan_field(vp, sd, fd, bsSlot, bfSlot, false, intraField, quality, plan);
    return plan;
}

std::vector<Span> frame_spans(const OutputFraming &g, const FieldMeta &slot0, bool slot0First,
                              const FieldMeta &slot1, bool slot1First, bool overcorrect)
{
    std::vector<Span> spans;
    const int32_t avs = g.activeVideoStart, ave = g.activeVideoStart + g.activeWidth;
    auto append = [&](const FieldMeta &f, bool isFirst) {
        const int32_t offset = isFirst ? 0 : 1;
        for (const Dropout &d : f.dropouts) {
            const int32_t frameRow = (2 * (d.fieldLine - 1)) + offset;
            const int32_t y = g.topPad + frameRow - g.firstActiveFrameLine;
            if (y < 0 || y >= g.height) continue;
            int32_t x0 = d.startx, x1 = d.endx;
            if (overcorrect) {
                const int32_t dots = 24;
                x0 = (x0 > dots) ? x0 - dots : 0;
                x1 = (x1 < g.fieldWidth - dots) ? x1 + dots : g.fieldWidth;
            }
            if (x0 < avs) x0 = avs;
            if (x1 > ave) x1 = ave;
            if (x1 <= x0) continue;
            spans.push_back({y, x0 - avs + g.leftPad, x1 - avs + g.leftPad, 0});
        }
    };
    append(slot0, slot0First);
    append(slot1, slot1First);
    std::sort(spans.begin(), spans.end(), [](const Span &a, const Span &b) {
        if (a.y != b.y) return a.y < b.y;
        if (a.x_start != b.x_start) return a.x_start < b.x_start;
        return a.x_end < b.x_end;
    });
    return spans;
}

}  // namespace chdg
