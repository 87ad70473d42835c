// Recursive-descent JSON reader (RFC 8259) with a nesting limit.
#include "json.h"

#include <cmath>
#include <cstdlib>
#include <cstring>

namespace mypbr_host {

const Json* Json::find(const std::string& key) const {
    if (kind != Object)
        return nullptr;
    for (const auto& m : members)
        if (m.first == key)
            return &m.second;
    return nullptr;
}

double Json::num(const std::string& key, double fallback) const {
    const Json* v = find(key);
    return v && v->kind == Number ? v->number : fallback;
}

long long Json::integer(const std::string& key, long long fallback) const {
    const Json* v = find(key);
    if (!v || v->kind != Number || !(std::fabs(v->number) < 9.0e15))
        return fallback;
    return (long long)v->number;
}

std::string Json::str(const std::string& key, const std::string& fallback) const {
    const Json* v = find(key);
    return v && v->kind == String ? v->text : fallback;
}

bool Json::flag(const std::string& key, bool fallback) const {
    const Json* v = find(key);
    return v && v->kind == Bool ? v->boolean : fallback;
}

namespace {

struct Reader {
    const char* p;
    const char* end;
    const char* begin;
    std::string error;

    bool fail(const std::string& what) {
        if (error.empty())
            error = what + " at byte " + std::to_string(p - begin);
        return false;
    }
    void blank() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r'))
            p++;
    }
    bool word(const char* w) {
        size_t n = std::strlen(w);
        if (size_t(end - p) < n || std::memcmp(p, w, n) != 0)
            return fail("unexpected text");
        p += n;
        return true;
    }
    static void put_utf8(std::string& s, unsigned cp) {
        if (cp < 0x80) {
            s += char(cp);
        } else if (cp < 0x800) {
            s += char(0xc0 | (cp >> 6));
            s += char(0x80 | (cp & 0x3f));
        } else if (cp < 0x10000) {
            s += char(0xe0 | (cp >> 12));
            s += char(0x80 | ((cp >> 6) & 0x3f));
            s += char(0x80 | (cp & 0x3f));
        } else {
            s += char(0xf0 | (cp >> 18));
            s += char(0x80 | ((cp >> 12) & 0x3f));
            s += char(0x80 | ((cp >> 6) & 0x3f));
            s += char(0x80 | (cp & 0x3f));
        }
    }
    bool hex4(unsigned& v) {
        if (end - p < 4)
            return fail("short \\u escape");
        v = 0;
        for (int k = 0; k < 4; k++) {
            char c = *p++;
            v <<= 4;
            if (c >= '0' && c <= '9')
                v |= unsigned(c - '0');
            else if (c >= 'a' && c <= 'f')
                v |= unsigned(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F')
                v |= unsigned(c - 'A' + 10);
            else
                return fail("bad \\u escape");
        }
        return true;
    }
    bool string(std::string& out) {
        p++;  // opening quote
        out.clear();
        while (true) {
            if (p >= end)
                return fail("unterminated string");
            char c = *p++;
            if (c == '"')
                return true;
            if ((unsigned char)c < 0x20)
                return fail("control character in string");
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p >= end)
                return fail("unterminated escape");
            char e = *p++;
            switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    unsigned cp = 0;
                    if (!hex4(cp))
                        return false;
                    if (cp >= 0xd800 && cp < 0xdc00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                        const char* save = p;
                        p += 2;
                        unsigned lo = 0;
                        if (!hex4(lo))
                            return false;
                        if (lo >= 0xdc00 && lo < 0xe000)
                            cp = 0x10000 + ((cp - 0xd800) << 10) + (lo - 0xdc00);
                        else
                            p = save;
                    }
                    put_utf8(out, cp);
                    break;
                }
                default: return fail("bad escape");
            }
        }
    }
    bool number(double& out) {
        const char* start = p;
        if (p < end && *p == '-')
            p++;
        if (p >= end || !(*p >= '0' && *p <= '9'))
            return fail("bad number");
        while (p < end && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '+' ||
                           *p == '-'))
            p++;
        std::string digits(start, p);
        char* stop = nullptr;
        out = std::strtod(digits.c_str(), &stop);
        if (!stop || *stop != '\0')
            return fail("bad number");
        return true;
    }
    bool value(Json& v, int depth) {
        if (depth > 200)
            return fail("nesting too deep");
        blank();
        if (p >= end)
            return fail("unexpected end");
        char c = *p;
        if (c == '{') {
            v.kind = Json::Object;
            p++;
            blank();
            if (p < end && *p == '}') {
                p++;
                return true;
            }
            while (true) {
                blank();
                if (p >= end || *p != '"')
                    return fail("expected a key");
                std::string key;
                if (!string(key))
                    return false;
                blank();
                if (p >= end || *p != ':')
                    return fail("expected ':'");
                p++;
                v.members.emplace_back(std::move(key), Json());
                if (!value(v.members.back().second, depth + 1))
                    return false;
                blank();
                if (p < end && *p == ',') {
                    p++;
                    continue;
                }
                if (p < end && *p == '}') {
                    p++;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = Json::Array;
            p++;
            blank();
            if (p < end && *p == ']') {
                p++;
                return true;
            }
            while (true) {
                v.items.emplace_back();
                if (!value(v.items.back(), depth + 1))
                    return false;
                blank();
                if (p < end && *p == ',') {
                    p++;
                    continue;
                }
                if (p < end && *p == ']') {
                    p++;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::String;
            return string(v.text);
        }
        if (c == 't') {
            v.kind = Json::Bool;
            v.boolean = true;
            return word("true");
        }
        if (c == 'f') {
            v.kind = Json::Bool;
            return word("false");
        }
        if (c == 'n') {
            v.kind = Json::Null;
            return word("null");
        }
        v.kind = Json::Number;
        return number(v.number);
    }
};

}  // namespace

bool parse_json(const char* text, size_t size, Json& out, std::string& error) {
    Reader r{text, text + size, text, {}};
    // a UTF-8 byte-order mark is tolerated
    if (size >= 3 && (unsigned char)text[0] == 0xef && (unsigned char)text[1] == 0xbb && (unsigned char)text[2] == 0xbf)
        r.p += 3;
    out = Json();
    if (!r.value(out, 0)) {
        error = r.error;
        return false;
    }
    r.blank();
    if (r.p != r.end) {
        error = "text after the JSON value at byte " + std::to_string(r.p - r.begin);
        return false;
    }
    return true;
}

}  // namespace mypbr_host
