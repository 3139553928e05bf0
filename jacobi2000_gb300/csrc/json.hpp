// A small JSON reader for config.json and safetensors headers: objects,
// arrays, strings (with escapes), numbers, true/false/null. Throws
// std::runtime_error on malformed input.
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace jc {

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;  // keeps file order

    const Json* find(const std::string& k) const {
        if (kind != Object) return nullptr;
        for (auto& kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
    const Json& at(const std::string& k) const {
        const Json* j = find(k);
        if (!j) throw std::runtime_error("missing field `" + k + "`");
        return *j;
    }
    double number() const {
        if (kind != Number) throw std::runtime_error("expected a number");
        return num;
    }
    long long integer() const {
        double v = number();
        if (v != (double)(long long)v) throw std::runtime_error("expected an integer");
        return (long long)v;
    }
    const std::string& string() const {
        if (kind != String) throw std::runtime_error("expected a string");
        return str;
    }

    static Json parse(const char* p, size_t n) {
        Parser ps{p, p + n};
        ps.ws();
        Json j = ps.value(0);
        ps.ws();
        if (ps.p != ps.e) throw std::runtime_error("trailing characters after JSON value");
        return j;
    }

   private:
    struct Parser {
        const char* p;
        const char* e;
        void ws() {
            while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
        }
        [[noreturn]] void fail(const char* what) { throw std::runtime_error(std::string("JSON: ") + what); }
        char peek() { return p < e ? *p : '\0'; }
        void expect(char c) {
            if (p >= e || *p != c) fail("unexpected character");
            p++;
        }
        Json value(int depth) {
            if (depth > 64) fail("nesting too deep");
            ws();
            char c = peek();
            Json j;
            if (c == '{') {
                j.kind = Object;
                p++;
                ws();
                if (peek() == '}') { p++; return j; }
                for (;;) {
                    ws();
                    Json k = string_value();
                    ws();
                    expect(':');
                    Json v = value(depth + 1);
                    j.obj.emplace_back(std::move(k.str), std::move(v));
                    ws();
                    if (peek() == ',') { p++; continue; }
                    expect('}');
                    return j;
                }
            }
            if (c == '[') {
                j.kind = Array;
                p++;
                ws();
                if (peek() == ']') { p++; return j; }
                for (;;) {
                    j.arr.push_back(value(depth + 1));
                    ws();
                    if (peek() == ',') { p++; continue; }
                    expect(']');
                    return j;
                }
            }
            if (c == '"') return string_value();
            if (c == 't' && e - p >= 4 && std::string(p, 4) == "true") { p += 4; j.kind = Bool; j.b = true; return j; }
            if (c == 'f' && e - p >= 5 && std::string(p, 5) == "false") { p += 5; j.kind = Bool; return j; }
            if (c == 'n' && e - p >= 4 && std::string(p, 4) == "null") { p += 4; return j; }
            if (c == '-' || (c >= '0' && c <= '9')) {
                const char* s = p;
                if (*p == '-') p++;
                while (p < e && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '+' ||
                                 *p == '-'))
                    p++;
                std::string tok(s, p);
                char* end = nullptr;
                j.kind = Number;
                j.num = std::strtod(tok.c_str(), &end);
                if (!end || *end != '\0') fail("bad number");
                return j;
            }
            fail("unexpected token");
        }
        Json string_value() {
            Json j;
            j.kind = String;
            expect('"');
            while (p < e && *p != '"') {
                char c = *p++;
                if (c == '\\') {
                    if (p >= e) fail("bad escape");
                    char x = *p++;
                    switch (x) {
                        case '"': j.str += '"'; break;
                        case '\\': j.str += '\\'; break;
                        case '/': j.str += '/'; break;
                        case 'b': j.str += '\b'; break;
                        case 'f': j.str += '\f'; break;
                        case 'n': j.str += '\n'; break;
                        case 'r': j.str += '\r'; break;
                        case 't': j.str += '\t'; break;
                        case 'u': {
                            if (e - p < 4) fail("bad \\u escape");
                            unsigned cp = (unsigned)std::strtoul(std::string(p, 4).c_str(), nullptr, 16);
                            p += 4;
                            if (cp < 0x80) j.str += (char)cp;
                            else if (cp < 0x800) { j.str += (char)(0xC0 | (cp >> 6)); j.str += (char)(0x80 | (cp & 0x3F)); }
                            else { j.str += (char)(0xE0 | (cp >> 12)); j.str += (char)(0x80 | ((cp >> 6) & 0x3F)); j.str += (char)(0x80 | (cp & 0x3F)); }
                            break;
                        }
                        default: fail("bad escape");
                    }
                } else {
                    j.str += c;
                }
            }
            expect('"');
            return j;
        }
    };
};

}  // namespace jc
