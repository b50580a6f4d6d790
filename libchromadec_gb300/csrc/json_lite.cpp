// json_lite.cpp -- recursive-descent JSON reader (RFC 8259 subset sufficient
// for ld-decode's .tbc.json sidecars; \u escapes decode to UTF-8).
#include "json_lite.h"

#include <cstdlib>
#include <cstring>

namespace chdg::json {

namespace {

struct Parser {
    const char *p, *end, *begin;
    std::string err;
    int depth = 0;

    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    }
    bool fail(const char *why)
    {
        if (err.empty()) err = "offset " + std::to_string(p - begin) + ": " + why;
        return false;
    }
    bool lit(const char *w)
    {
        const size_t n = std::strlen(w);
        if ((size_t)(end - p) < n || std::strncmp(p, w, n) != 0) return fail("bad literal");
        p += n;
        return true;
    }
    static void put_utf8(std::string &s, unsigned cp)
    {
        if (cp < 0x80) s += (char)cp;
        else if (cp < 0x800) { s += (char)(0xC0 | (cp >> 6)); s += (char)(0x80 | (cp & 0x3F)); }
        else if (cp < 0x10000) {
            s += (char)(0xE0 | (cp >> 12)); s += (char)(0x80 | ((cp >> 6) & 0x3F)); s += (char)(0x80 | (cp & 0x3F));
        } else {
            s += (char)(0xF0 | (cp >> 18)); s += (char)(0x80 | ((cp >> 12) & 0x3F));
            s += (char)(0x80 | ((cp >> 6) & 0x3F)); s += (char)(0x80 | (cp & 0x3F));
        }
    }
    bool hex4(unsigned &v)
    {
        if (end - p < 4) return fail("short \\u escape");
        v = 0;
        for (int i = 0; i < 4; i++) {
            const char c = *p++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }
    bool string(std::string &s)
    {
        if (p >= end || *p != '"') return fail("expected string");
        p++;
        while (p < end && *p != '"') {
            char c = *p++;
            if (c == '\\') {
                if (p >= end) return fail("bad escape");
                c = *p++;
                switch (c) {
                case '"': s += '"'; break;
                case '\\': s += '\\'; break;
                case '/': s += '/'; break;
                case 'b': s += '\b'; break;
                case 'f': s += '\f'; break;
                case 'n': s += '\n'; break;
                case 'r': s += '\r'; break;
                case 't': s += '\t'; break;
                case 'u': {
                    unsigned cp;
                    if (!hex4(cp)) return false;
                    if (cp >= 0xD800 && cp < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                        p += 2;
                        unsigned lo;
                        if (!hex4(lo)) return false;
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    put_utf8(s, cp);
                    break;
                }
                default: return fail("bad escape");
                }
            } else {
                s += c;
            }
        }
        if (p >= end) return fail("unterminated string");
        p++;
        return true;
    }
    bool value(Value &v)
    {
        if (++depth > 256) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        bool ok = true;
        switch (*p) {
        case '{': {
            v.kind = Value::Object;
            p++;
            ws();
            if (p < end && *p == '}') { p++; break; }
            for (;;) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (p >= end || *p != ':') return fail("expected ':'");
                p++;
                Value child;
                if (!value(child)) return false;
                v.obj[k] = std::move(child);
                ws();
                if (p < end && *p == ',') { p++; continue; }
                if (p < end && *p == '}') { p++; break; }
                return fail("expected ',' or '}'");
            }
            break;
        }
        case '[': {
            v.kind = Value::Array;
            p++;
            ws();
            if (p < end && *p == ']') { p++; break; }
            for (;;) {
                Value child;
                if (!value(child)) return false;
                v.arr.push_back(std::move(child));
                ws();
                if (p < end && *p == ',') { p++; continue; }
                if (p < end && *p == ']') { p++; break; }
                return fail("expected ',' or ']'");
            }
            break;
        }
        case '"':
            v.kind = Value::String;
            ok = string(v.str);
            break;
        case 't': v.kind = Value::Bool; v.b = true; ok = lit("true"); break;
        case 'f': v.kind = Value::Bool; v.b = false; ok = lit("false"); break;
        case 'n': v.kind = Value::Null; ok = lit("null"); break;
        default: {
            char *e = nullptr;
            std::string tok;
            const char *q = p;
            while (q < end && (std::strchr("+-0123456789.eE", *q) != nullptr)) q++;
            tok.assign(p, q);
            if (tok.empty()) return fail("unexpected character");
            v.kind = Value::Number;
            v.num = std::strtod(tok.c_str(), &e);
            if (e == nullptr || *e != '\0') return fail("bad number");
            p = q;
        }
        }
        depth--;
        return ok;
    }
};

}  // namespace

bool parse(const std::string &text, Value &out, std::string &err)
{
    Parser ps{text.data(), text.data() + text.size(), text.data(), {}};
    if (!ps.value(out)) {
        err = ps.err;
        return false;
    }
    ps.ws();
    if (ps.p != ps.end) {
        ps.fail("trailing characters");
        err = ps.err;
        return false;
    }
    return true;
}

}  // namespace chdg::json
