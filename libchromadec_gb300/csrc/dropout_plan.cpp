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
    int32_t source = 0;
    double quality = -1.0;
    int32_t distance = 0;
};

// Every source's share of one frame: index 0 is the primary.
struct Sources {
    std::vector<const VideoParams *> vp;
    std::vector<std::vector<DLoc>> first, second;   // located dropouts, broadcast / pairing order
    std::vector<double> quality;
};

// findPotentialReplacementLine, dropout_corrector.cpp:417-466 (vp: the
// source's video parameters)
void find_potential(const VideoParams &vp, const std::vector<DLoc> &target, size_t ti,
                    const std::vector<DLoc> &source, bool sameField, int32_t offset, int32_t step, int32_t sourceNo,
                    double quality, std::vector<Rep> &cands)
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
            r.source = sourceNo;
            r.quality = quality;
            cands.push_back(r);
            return;
        }
    }
}

// findReplacementLine, dropout_corrector.cpp:248-414: every source in turn
// (this field up and down, then the other field), nearest frame line first,
// the higher quality among equally near candidates. thisD / otherD are the
// per-source lists of this field and the other; the target is thisD[0][idx].
Rep find_replacement(const VideoParams &vp, const Sources &S, const std::vector<std::vector<DLoc>> &thisD,
                     const std::vector<std::vector<DLoc>> &otherD, size_t idx, bool thisFieldIsFirst,
                     bool matchChromaPhase, bool isColourBurst, bool intraField)
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
    const std::vector<DLoc> &target = thisD[0];
    for (size_t s = 0; s < thisD.size(); s++) {
        const VideoParams &sv = *S.vp[s];
        const double q = S.quality[s];
        find_potential(sv, target, idx, thisD[s], true, 0, -step, (int32_t)s, q, cands);
        find_potential(sv, target, idx, thisD[s], true, step, step, (int32_t)s, q, cands);
        if (!isColourBurst && !intraField) {
            find_potential(sv, target, idx, otherD[s], false, otherOffset, -step, (int32_t)s, q, cands);
            find_potential(sv, target, idx, otherD[s], false, otherOffset + step, step, (int32_t)s, q, cands);
        }
    }
    Rep rep;
    if (!cands.empty()) {
        rep.distance = 1000000;
        rep.quality = -1;
        for (const Rep &c : cands) {
            const int32_t dropLine = (2 * target[idx].fieldLine) + (thisFieldIsFirst ? 0 : 1);
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
// (dropout_corrector.cpp:117-157, 469-530). A replacement from source s >= 1
// reads that source's field of the same or the other parity: plan.extras
// holds each extra source's first and second field at 2(s-1) and 2(s-1)+1.
void plan_field(const VideoParams &vp, const Sources &S, const std::vector<std::vector<DLoc>> &thisD,
                const std::vector<std::vector<DLoc>> &otherD, int thisSlot, int otherSlot, bool thisFieldIsFirst,
                bool intraField, FramePlan &plan)
{
    auto where = [&](const Rep &r, int32_t &slot, int32_t &extra) {
        slot = r.sameField ? thisSlot : otherSlot;
        extra = -1;
        if (r.source > 0) {
            const bool first = (r.sameField == thisFieldIsFirst);   // the extra's first-field list
            extra = 2 * (r.source - 1) + (first ? 0 : 1);
        }
    };
    const std::vector<DLoc> &target = thisD[0];
    for (size_t i = 0; i < target.size(); i++) {
        Rep rep, crep;
        if (target[i].location == BURST)
            rep = find_replacement(vp, S, thisD, otherD, i, thisFieldIsFirst, true, true, intraField);
        if (target[i].location == VISIBLE) {
            rep = find_replacement(vp, S, thisD, otherD, i, thisFieldIsFirst, false, false, intraField);
            crep = find_replacement(vp, S, thisD, otherD, i, thisFieldIsFirst, true, false, intraField);
        }
        if (rep.fieldLine == -1) {
            plan.failed++;
            continue;
        }
        plan.corrected++;
        plan.totalDistance += rep.distance;
        DropOp op{};
        op.field = thisSlot;
        op.line = target[i].fieldLine - 1;
        op.startx = target[i].startx;
        op.endx = target[i].endx;
        where(rep, op.srcField, op.srcExtra);
        op.srcLine = rep.fieldLine - 1;
        op.chrExtra = -1;
        if (crep.fieldLine == -1 || (target[i].fieldLine == rep.fieldLine && target[i].fieldLine == crep.fieldLine)) {
            op.mode = 1;
        } else {
            op.mode = 2;
            where(crep, op.chrField, op.chrExtra);
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
                     bool intraField, const std::vector<ExtraFrame> &extras)
{
    FramePlan plan;
    // broadcast order (dropout_corrector.cpp:56-57)
    const bool s0first = slot0.isFirstField;
    const FieldMeta &bf = s0first ? slot0 : slot1;
    const FieldMeta &bs = s0first ? slot1 : slot0;
    const int bfSlot = s0first ? 0 : 1, bsSlot = s0first ? 1 : 0;
    if (bf.dropouts.empty() && bs.dropouts.empty()) return plan;
    // sources: the primary, then the extras (dropout_corrector.cpp:60-103)
    const size_t n = 1 + extras.size();
    Sources S;
    S.vp.assign(n, &vp);
    S.first.assign(n, {});
    S.second.assign(n, {});
    S.quality.assign(n, 0.0);
    S.quality[0] = (bf.bPSNR + bs.bPSNR) / 2.0;
    auto locate = [&](const VideoParams &svp, const FieldMeta &f, std::vector<DLoc> &out) {
        if (f.dropouts.empty()) return;
        out = populate(svp, f, overcorrect);
        set_locations(vp, out);   // the corrector's own (primary) video parameters
    };
    locate(vp, bf, S.first[0]);
    locate(vp, bs, S.second[0]);
    for (size_t e = 0; e < extras.size(); e++) {
        S.vp[e + 1] = &extras[e].vp;
        S.quality[e + 1] = extras[e].quality;
        locate(extras[e].vp, extras[e].first, S.first[e + 1]);
        locate(extras[e].vp, extras[e].second, S.second[e + 1]);
        plan.extras.push_back(extras[e].firstField);
        plan.extras.push_back(extras[e].secondField);
    }
    plan_field(vp, S, S.first, S.second, bfSlot, bsSlot, true, intraField, plan);
    plan_field(vp, S, S.second, S.first, bsSlot, bfSlot, false, intraField, plan);
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
