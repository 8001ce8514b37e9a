// Minimal JSON reader for glTF documents: a DOM of values, strict parsing,
// nesting depth limit, \u escapes (with surrogate pairs) decoded to UTF-8.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace swr {
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;

    const Value* get(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    const Value* at(size_t i) const { return kind == Array && i < arr.size() ? &arr[i] : nullptr; }
    size_t size() const { return kind == Array ? arr.size() : (kind == Object ? obj.size() : 0); }
    bool is_num() const { return kind == Number; }
    double num_or(double d) const { return kind == Number ? num : d; }
};

// Convenience lookups on a possibly-null value.
inline const Value* get(const Value* v, const char* key) { return v ? v->get(key) : nullptr; }
inline double num(const Value* v, double d) { return v ? v->num_or(d) : d; }
// Out-of-range and non-finite numbers give INT64_MIN, which every index,
// count and offset check rejects.
inline int64_t integer(const Value* v, int64_t d) {
    if (!v || v->kind != Value::Number) return d;
    if (!(v->num >= -9.0e18 && v->num <= 9.0e18)) return INT64_MIN;
    return (int64_t)v->num;
}
inline std::string string(const Value* v, const char* d = "") {
    return (v && v->kind == Value::String) ? v->str : std::string(d);
}

class Parser {
public:
    Parser(const char* p, size_t n) : p_(p), end_(p + n) {}

    bool parse(Value& out, std::string& err) {
        ws();
        if (!value(out, 0)) {
            err = err_.empty() ? "malformed JSON" : err_;
            return false;
        }
        ws();
        if (p_ != end_) {
            err = "trailing characters after JSON value";
            return false;
        }
        return true;
    }

private:
    const char* p_;
    const char* end_;
    std::string err_;

    bool fail(const char* m) {
        if (err_.empty()) err_ = m;
        return false;
    }
    void ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if ((size_t)(end_ - p_) < n || std::memcmp(p_, s, n) != 0) return false;
        p_ += n;
        return true;
    }
    static void put_utf8(std::string& o, uint32_t c) {
        if (c < 0x80) {
            o += (char)c;
        } else if (c < 0x800) {
            o += (char)(0xC0 | (c >> 6));
            o += (char)(0x80 | (c & 0x3F));
        } else if (c < 0x10000) {
            o += (char)(0xE0 | (c >> 12));
            o += (char)(0x80 | ((c >> 6) & 0x3F));
            o += (char)(0x80 | (c & 0x3F));
        } else {
            o += (char)(0xF0 | (c >> 18));
            o += (char)(0x80 | ((c >> 12) & 0x3F));
            o += (char)(0x80 | ((c >> 6) & 0x3F));
            o += (char)(0x80 | (c & 0x3F));
        }
    }
    bool hex4(uint32_t& v) {
        if (end_ - p_ < 4) return fail("truncated \\u escape");
        v = 0;
        for (int i = 0; i < 4; ++i) {
            const char c = *p_++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }
    bool string_(std::string& o) {
        ++p_;  // opening quote
        while (p_ < end_) {
            const char c = *p_++;
            if (c == '"') return true;
            if ((unsigned char)c < 0x20) return fail("control character in string");
            if (c != '\\') {
                o += c;
                continue;
            }
            if (p_ >= end_) break;
            const char e = *p_++;
            switch (e) {
                case '"': o += '"'; break;
                case '\\': o += '\\'; break;
                case '/': o += '/'; break;
                case 'b': o += '\b'; break;
                case 'f': o += '\f'; break;
                case 'n': o += '\n'; break;
                case 'r': o += '\r'; break;
                case 't': o += '\t'; break;
                case 'u': {
                    uint32_t c1;
                    if (!hex4(c1)) return false;
                    if (c1 >= 0xD800 && c1 < 0xDC00) {
                        uint32_t c2;
                        if (!(lit("\\u") && hex4(c2)) || c2 < 0xDC00 || c2 >= 0xE000)
                            return fail("unpaired surrogate");
                        c1 = 0x10000 + ((c1 - 0xD800) << 10) + (c2 - 0xDC00);
                    } else if (c1 >= 0xDC00 && c1 < 0xE000) {
                        return fail("unpaired surrogate");
                    }
                    put_utf8(o, c1);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        return fail("unterminated string");
    }
    bool number_(double& d) {
        const char* s = p_;
        if (p_ < end_ && *p_ == '-') ++p_;
        if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) return fail("bad number");
        while (p_ < end_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' || *p_ == '+' ||
                             *p_ == '-'))
            ++p_;
        const std::string t(s, p_);
        char* e = nullptr;
        d = std::strtod(t.c_str(), &e);
        if (!e || *e != '\0') return fail("bad number");
        return true;
    }
    bool value(Value& v, int depth) {
        if (depth > 256) return fail("JSON nested too deeply");
        if (p_ >= end_) return fail("unexpected end of JSON");
        const char c = *p_;
        if (c == '{') {
            v.kind = Value::Object;
            ++p_;
            ws();
            if (p_ < end_ && *p_ == '}') {
                ++p_;
                return true;
            }
            for (;;) {
                ws();
                if (p_ >= end_ || *p_ != '"') return fail("expected object key");
                std::string k;
                if (!string_(k)) return false;
                ws();
                if (p_ >= end_ || *p_ != ':') return fail("expected ':'");
                ++p_;
                ws();
                v.obj.emplace_back(std::move(k), Value());
                if (!value(v.obj.back().second, depth + 1)) return false;
                ws();
                if (p_ < end_ && *p_ == ',') {
                    ++p_;
                    continue;
                }
                if (p_ < end_ && *p_ == '}') {
                    ++p_;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = Value::Array;
            ++p_;
            ws();
            if (p_ < end_ && *p_ == ']') {
                ++p_;
                return true;
            }
            for (;;) {
                ws();
                v.arr.emplace_back();
                if (!value(v.arr.back(), depth + 1)) return false;
                ws();
                if (p_ < end_ && *p_ == ',') {
                    ++p_;
                    continue;
                }
                if (p_ < end_ && *p_ == ']') {
                    ++p_;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Value::String;
            return string_(v.str);
        }
        if (lit("true")) {
            v.kind = Value::Bool;
            v.b = true;
            return true;
        }
        if (lit("false")) {
            v.kind = Value::Bool;
            v.b = false;
            return true;
        }
        if (lit("null")) {
            v.kind = Value::Null;
            return true;
        }
        v.kind = Value::Number;
        return number_(v.num);
    }
};

}  // namespace json
}  // namespace swr
