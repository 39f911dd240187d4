// json.cpp — recursive-descent JSON parser (RFC 8259).
#include "json.h"

#include <cmath>
#include <cstdlib>
#include <cstring>

namespace aq {
namespace {

struct Parser {
    const char* s;
    size_t n, i = 0;
    int depth = 0;

    [[noreturn]] void fail(const char* what) {
        throw JsonError(std::string("JSON parse error at byte ") + std::to_string(i) + ": " + what);
    }
    void ws() {
        while (i < n && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) ++i;
    }
    bool lit(const char* w) {
        size_t l = strlen(w);
        if (i + l <= n && memcmp(s + i, w, l) == 0) { i += l; return true; }
        return false;
    }
    static void put_utf8(std::string& out, unsigned cp) {
        if (cp < 0x80) out += (char)cp;
        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
        else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18)); out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F));
        }
    }
    unsigned hex4() {
        if (i + 4 > n) fail("truncated \\u escape");
        unsigned v = 0;
        for (int k = 0; k < 4; ++k) {
            char c = s[i++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
            else fail("bad hex digit");
        }
        return v;
    }
    std::string string() {
        if (s[i] != '"') fail("expected '\"'");
        ++i;
        std::string out;
        while (true) {
            if (i >= n) fail("unterminated string");
            char c = s[i++];
            if (c == '"') break;
            if ((unsigned char)c < 0x20) fail("control character in string");
            if (c != '\\') { out += c; continue; }
            if (i >= n) fail("unterminated escape");
            char e = s[i++];
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
                    unsigned cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00) {
                        if (!(i + 1 < n && s[i] == '\\' && s[i + 1] == 'u')) fail("lone surrogate");
                        i += 2;
                        unsigned lo = hex4();
                        if (lo < 0xDC00 || lo >= 0xE000) fail("bad low surrogate");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    put_utf8(out, cp);
                    break;
                }
                default: fail("bad escape");
            }
        }
        return out;
    }
    double number() {
        size_t st = i;
        if (s[i] == '-') ++i;
        if (i >= n) fail("truncated number");
        if (s[i] == '0') ++i;
        else if (s[i] >= '1' && s[i] <= '9') while (i < n && s[i] >= '0' && s[i] <= '9') ++i;
        else fail("bad number");
        if (i < n && s[i] == '.') {
            ++i;
            if (!(i < n && s[i] >= '0' && s[i] <= '9')) fail("bad fraction");
            while (i < n && s[i] >= '0' && s[i] <= '9') ++i;
        }
        if (i < n && (s[i] == 'e' || s[i] == 'E')) {
            ++i;
            if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
            if (!(i < n && s[i] >= '0' && s[i] <= '9')) fail("bad exponent");
            while (i < n && s[i] >= '0' && s[i] <= '9') ++i;
        }
        std::string tok(s + st, i - st);
        const double v = strtod(tok.c_str(), nullptr);
        if (!std::isfinite(v)) fail("number out of range");
        return v;
    }
    Json value() {
        if (++depth > 256) fail("nesting too deep");
        ws();
        if (i >= n) fail("unexpected end of input");
        Json j;
        char c = s[i];
        if (c == '{') {
            j.kind = Json::Object;
            ++i; ws();
            if (i < n && s[i] == '}') { ++i; --depth; return j; }
            while (true) {
                ws();
                if (i >= n) fail("unterminated object");
                std::string k = string();
                ws();
                if (i >= n || s[i] != ':') fail("expected ':'");
                ++i;
                Json v = value();
                j.obj.emplace_back(std::move(k), std::move(v));
                ws();
                if (i < n && s[i] == ',') { ++i; continue; }
                if (i < n && s[i] == '}') { ++i; break; }
                fail("expected ',' or '}'");
            }
        } else if (c == '[') {
            j.kind = Json::Array;
            ++i; ws();
            if (i < n && s[i] == ']') { ++i; --depth; return j; }
            while (true) {
                j.arr.push_back(value());
                ws();
                if (i < n && s[i] == ',') { ++i; continue; }
                if (i < n && s[i] == ']') { ++i; break; }
                fail("expected ',' or ']'");
            }
        } else if (c == '"') {
            j.kind = Json::String;
            j.str = string();
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            j.kind = Json::Number;
            j.num = number();
        } else if (lit("true")) {
            j.kind = Json::Bool; j.b = true;
        } else if (lit("false")) {
            j.kind = Json::Bool; j.b = false;
        } else if (lit("null")) {
            j.kind = Json::Null;
        } else {
            fail("unexpected character");
        }
        --depth;
        return j;
    }
};

}  // namespace

Json json_parse(const std::string& text) {
    Parser p{text.data(), text.size()};
    Json j = p.value();
    p.ws();
    if (p.i != p.n) p.fail("trailing characters");
    return j;
}

}  // namespace aq
