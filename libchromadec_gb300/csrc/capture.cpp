// capture.cpp -- ld-decode .tbc + JSON sidecar reader.
//
// The sidecar keys and the system defaults applied after reading follow the
// reference's LdDecodeMetaData (src/metadata/ld_metadata_json.cpp:64-119,
// 232-260; defaults src/metadata/core.cpp:40-86, 743-810); the field pairing
// follows src/metadata/core.cpp:1092-1190.
#include "capture.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstring>
#include <fstream>
#include <sstream>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <chromadec/errors.h>

#include "error_state.h"
#include "json_lite.h"

namespace chdg {

namespace {

int fail(int status, const std::string &msg)
{
    chd::detail::set_last_error("chd_video_open_composite: " + msg);
    return status;
}

bool file_exists(const std::string &p)
{
    struct stat st;
    return ::stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

std::string normalise_system(std::string s)
{
    while (!s.empty() && std::isspace((unsigned char)s.front())) s.erase(s.begin());
    while (!s.empty() && std::isspace((unsigned char)s.back())) s.pop_back();
    for (auto &c : s) {
        if (c == '-' || c == ' ') c = '_';
        c = (char)std::toupper((unsigned char)c);
    }
    return s;
}

// parseVideoSystemName (src/metadata/core.cpp:116-159)
bool parse_system(const std::string &name, int &sys)
{
    const std::string n = normalise_system(name);
    if (n == "PAL" || n == "PALN" || n == "PAL_N" || n == "405" || n == "819") { sys = SYS_PAL; return true; }
    if (n == "NTSC" || n == "NTSCJ" || n == "NTSC_J") { sys = SYS_NTSC; return true; }
    if (n == "PAL_M" || n == "MPAL" || n == "PALM" || n == "N_LINHA" || n == "NLINHA" || n == "PAL_N_LINHA" ||
        n == "PAL_NLINHA") { sys = SYS_PAL_M; return true; }
    if (n == "SECAM" || n == "MESECAM" || n == "ME_SECAM") { sys = SYS_SECAM; return true; }
    return false;
}

int json_int(const json::Value *v, int dflt)
{
    return (v && v->is_number()) ? (int)v->num : dflt;
}

}  // namespace

Capture::~Capture()
{
    if (map_ != nullptr && map_ != MAP_FAILED) ::munmap(map_, mapBytes_);
    if (fd_ >= 0) ::close(fd_);
}

int Capture::open(const char *path, const char *meta_or_null, const chd_video_params_t *ovr)
{
    path_ = path;
    if (!file_exists(path_)) return fail(CHD_E_FILE_NOT_FOUND, std::string("file does not exist: ") + path);
    std::string meta;
    if (meta_or_null != nullptr) {
        meta = meta_or_null;
        if (!file_exists(meta)) return fail(CHD_E_FILE_NOT_FOUND, "sidecar does not exist: " + meta);
    } else if (file_exists(path_ + ".json")) {
        meta = path_ + ".json";
    } else if (file_exists(path_ + ".db")) {
        return fail(CHD_E_FORMAT_UNSUPPORTED, "SQLite sidecars (" + path_ + ".db) are not read by this build");
    } else {
        return fail(CHD_E_METADATA_MISSING, "no sidecar next to " + path_);
    }
    if (meta.size() >= 3 && meta.compare(meta.size() - 3, 3, ".db") == 0)
        return fail(CHD_E_FORMAT_UNSUPPORTED, "SQLite sidecars are not read by this build");

    std::ifstream in(meta, std::ios::binary);
    if (!in) return fail(CHD_E_IO, "cannot read " + meta);
    std::stringstream ss;
    ss << in.rdbuf();
    json::Value root;
    std::string err;
    if (!json::parse(ss.str(), root, err) || root.kind != json::Value::Object)
        return fail(CHD_E_METADATA_CORRUPT, meta + ": " + (err.empty() ? "not a JSON object" : err));
    const json::Value *v = root.get("videoParameters");
    if (v == nullptr || v->kind != json::Value::Object)
        return fail(CHD_E_METADATA_CORRUPT, meta + ": no videoParameters");

    // VideoParameters::read(JsonReader&), ld_metadata_json.cpp:64-119
    vp_.activeVideoEnd = json_int(v->get("activeVideoEnd"), -1);
    vp_.activeVideoStart = json_int(v->get("activeVideoStart"), -1);
    vp_.black16bIre = json_int(v->get("black16bIre"), -1);
    vp_.blanking16bIre = json_int(v->get("blanking16bIre"), -1);
    vp_.colourBurstEnd = json_int(v->get("colourBurstEnd"), -1);
    vp_.colourBurstStart = json_int(v->get("colourBurstStart"), -1);
    vp_.fieldHeight = json_int(v->get("fieldHeight"), -1);
    vp_.fieldWidth = json_int(v->get("fieldWidth"), -1);
    vp_.white16bIre = json_int(v->get("white16bIre"), -1);
    vp_.numberOfSequentialFields = json_int(v->get("numberOfSequentialFields"), -1);
    if (const json::Value *x = v->get("sampleRate"); x && x->is_number()) vp_.sampleRate = x->num;
    if (const json::Value *x = v->get("isSubcarrierLocked"); x && x->kind == json::Value::Bool)
        vp_.isSubcarrierLocked = x->b;
    if (const json::Value *x = v->get("isWidescreen"); x && x->kind == json::Value::Bool) vp_.isWidescreen = x->b;
    bool isSourcePal = false;
    if (const json::Value *x = v->get("isSourcePal"); x && x->kind == json::Value::Bool) isSourcePal = x->b;
    const json::Value *sys = v->get("system");
    if (sys == nullptr || sys->kind != json::Value::String || sys->str.empty()) {
        vp_.system = isSourcePal ? (vp_.fieldHeight < 300 ? SYS_PAL_M : SYS_PAL) : SYS_NTSC;
    } else if (!parse_system(sys->str, vp_.system)) {
        return fail(CHD_E_METADATA_CORRUPT, meta + ": unknown value for videoParameters.system");
    }
    if (vp_.blanking16bIre == -1) vp_.blanking16bIre = vp_.black16bIre;
    if (vp_.fieldWidth <= 0 || vp_.fieldHeight <= 0)
        return fail(CHD_E_METADATA_CORRUPT, meta + ": missing field geometry");

    // Open-time override: colour standard re-declaration and field order
    // (include/chromadec/video.h:18-29).
    firstFieldFirst_ = true;
    if (ovr != nullptr) {
        if (ovr->standard == CHD_STD_PAL) vp_.system = SYS_PAL;
        else if (ovr->standard == CHD_STD_PAL_M) vp_.system = SYS_PAL_M;
        else if (ovr->standard == CHD_STD_NTSC) vp_.system = SYS_NTSC;
        else if (ovr->standard == CHD_STD_SECAM) vp_.system = SYS_SECAM;
        if (ovr->is_second_field_first) firstFieldFirst_ = false;
        if (ovr->is_subcarrier_locked) vp_.isSubcarrierLocked = true;
    }
    // System defaults: fSC and the active frame lines (core.cpp:40-86, 743-810)
    switch (vp_.system) {
    case SYS_PAL: vp_.fSC = (283.75 * 15625) + 25; vp_.firstActiveFrameLine = 44; vp_.lastActiveFrameLine = 619; break;
    case SYS_NTSC: vp_.fSC = 315.0e6 / 88.0; vp_.firstActiveFrameLine = 39; vp_.lastActiveFrameLine = 524; break;
    case SYS_PAL_M:
        vp_.fSC = 5.0e6 * (63.0 / 88.0) * (909.0 / 910.0);
        vp_.firstActiveFrameLine = 39;
        vp_.lastActiveFrameLine = 524;
        break;
    default: vp_.fSC = 4286000.0; vp_.firstActiveFrameLine = 44; vp_.lastActiveFrameLine = 619; break;
    }

    // Fields (Field::read(JsonReader&), ld_metadata_json.cpp:232-260)
    if (const json::Value *fa = root.get("fields"); fa && fa->kind == json::Value::Array) {
        fields_.reserve(fa->arr.size());
        for (const auto &fv : fa->arr) {
            FieldMeta fm;
            if (const json::Value *x = fv.get("isFirstField"); x && x->kind == json::Value::Bool) fm.isFirstField = x->b;
            if (const json::Value *x = fv.get("pad"); x && x->kind == json::Value::Bool) fm.pad = x->b;
            if (const json::Value *vm = fv.get("vitsMetrics"))
                if (const json::Value *b = vm->get("bPSNR"); b && b->is_number()) fm.bPSNR = b->num;
            // Vbi::read (ld_metadata_json.cpp:34-56): up to 3 values, the rest 0
            if (const json::Value *vb = fv.get("vbi"))
                if (const json::Value *vd = vb->get("vbiData"); vd && vd->kind == json::Value::Array)
                    for (size_t i = 0; i < 3; i++)
                        fm.vbi[i] = (i < vd->arr.size()) ? (int32_t)vd->arr[i].num : 0;
            if (const json::Value *d = fv.get("dropOuts"); d && d->kind == json::Value::Object) {
                const json::Value *sx = d->get("startx"), *ex = d->get("endx"), *fl = d->get("fieldLine");
                const size_t n = sx && sx->kind == json::Value::Array ? sx->arr.size() : 0;
                if (!ex || !fl || ex->arr.size() != n || fl->arr.size() != n)
                    return fail(CHD_E_METADATA_CORRUPT, meta + ": dropout array sizes do not match");
                for (size_t i = 0; i < n; i++)
                    fm.dropouts.push_back({(int32_t)sx->arr[i].num, (int32_t)ex->arr[i].num, (int32_t)fl->arr[i].num});
            }
            fields_.push_back(std::move(fm));
        }
    }

    fd_ = ::open(path, O_RDONLY);
    if (fd_ < 0) return fail(CHD_E_IO, std::string("cannot open ") + path + ": " + std::strerror(errno));
    struct stat st;
    if (::fstat(fd_, &st) != 0) return fail(CHD_E_IO, "fstat failed");
    mapBytes_ = (size_t)st.st_size;
    const size_t fbytes = fieldLen() * 2;
    nsource_ = (int)(mapBytes_ / fbytes);
    if (mapBytes_ > 0) {
        map_ = ::mmap(nullptr, mapBytes_, PROT_READ, MAP_SHARED, fd_, 0);
        if (map_ == MAP_FAILED) {
            map_ = nullptr;
            return fail(CHD_E_IO, "mmap failed");
        }
        ::madvise(map_, mapBytes_, MADV_SEQUENTIAL);
    }
    return CHD_OK;
}

const FieldMeta &Capture::field(int seq) const
{
    static const FieldMeta empty{};
    if (seq < 1 || seq > (int)fields_.size()) return empty;
    return fields_[(size_t)seq - 1];
}

const uint16_t *Capture::fieldData(int seq) const
{
    if (seq < 1 || seq > nsource_ || map_ == nullptr) return nullptr;
    return static_cast<const uint16_t *>(map_) + fieldLen() * (size_t)(seq - 1);
}

int Capture::numFrames(bool firstFieldFirst) const
{
    int frameOffset = 0;
    if (firstFieldFirst) {
        if (!field(1).isFirstField) frameOffset = 1;
    } else {
        if (field(1).isFirstField) frameOffset = 1;
    }
    return (numMetadataFields() / 2) - frameOffset;
}

int Capture::fieldNumber(int frameNumber, int which, bool firstFieldFirst) const
{
    if (frameNumber < 1) return -1;
    int first, second;
    if (firstFieldFirst) {
        first = (frameNumber * 2) - 1;
        second = first + 1;
    } else {
        second = (frameNumber * 2) - 1;
        first = second + 1;
    }
    const int n = numMetadataFields();
    while (!field(first).isFirstField) {
        first++;
        second++;
        if (first > n || second > n) {
            first = second = -1;
            break;
        }
    }
    if (first > n || second > n) first = second = -1;
    if (first == -1) return -1;
    return which == 1 ? first : second;
}

void Capture::windowFrame(int frameNumber, bool firstFieldFirst, WindowField out[2]) const
{
    const int numInputFrames = numFrames(firstFieldFirst);
    const int nMeta = numMetadataFields();
    bool useBlank = frameNumber < 1 || frameNumber > numInputFrames;
    int metaFrame = useBlank ? 1 : frameNumber;
    int first = fieldNumber(metaFrame, 1, firstFieldFirst);
    int second = fieldNumber(metaFrame, 2, firstFieldFirst);
    auto metaSafe = [nMeta](int a, int b) { return a >= 1 && b >= 1 && a <= nMeta && b <= nMeta; };
    bool metaInvalid = !metaSafe(first, second);
    const bool srcInvalid = (first > nsource_ || second > nsource_);
    if (!useBlank && (metaInvalid || srcInvalid)) {
        useBlank = true;
        metaFrame = 1;
        first = fieldNumber(metaFrame, 1, firstFieldFirst);
        second = fieldNumber(metaFrame, 2, firstFieldFirst);
        metaInvalid = !metaSafe(first, second);
    }
    if (!metaInvalid) {
        out[0].isFirstField = field(first).isFirstField;
        out[1].isFirstField = field(second).isFirstField;
    } else {
        out[0].isFirstField = true;
        out[1].isFirstField = false;
        useBlank = true;
    }
    out[0].fieldNumber = metaInvalid ? 0 : first;
    out[1].fieldNumber = metaInvalid ? 0 : second;
    out[0].isPadding = out[1].isPadding = useBlank;
    out[0].source = useBlank ? 0 : first;
    out[1].source = useBlank ? 0 : second;
}

}  // namespace chdg
