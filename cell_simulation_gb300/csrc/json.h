// json.h — small recursive-descent JSON reader for the saved_models model
// format (src/simulation.rs:210-356 reads it through serde_json).  Objects
// keep their keys in a std::map, i.e. sorted by byte order, which is the
// iteration order serde_json uses without its `preserve_order` feature.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cellsim {

struct JsonValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    bool is_integer = false;  // number literal had no fraction/exponent
    std::string str;
    std::vector<JsonValue> arr;
    std::map<std::string, JsonValue> obj;

    bool has(const std::string& k) const { return kind == Object && obj.count(k) && obj.at(k).kind != Null; }
    const JsonValue& at(const std::string& k) const {
        if (kind != Object) throw std::runtime_error("JSON: expected an object when reading '" + k + "'");
        auto it = obj.find(k);
        if (it == obj.end()) throw std::runtime_error("JSON: missing key '" + k + "'");
        return it->second;
    }
    double as_number(const std::string& what) const {
        if (kind != Number) throw std::runtime_error("JSON: '" + what + "' must be a number");
        return num;
    }
    uint64_t as_u64(const std::string& what) const {
        if (kind != Number || !is_integer || num < 0) throw std::runtime_error("JSON: '" + what + "' must be a non-negative integer");
        return (uint64_t)num;
    }
    bool as_bool(const std::string& what) const {
        if (kind != Bool) throw std::runtime_error("JSON: '" + what + "' must be a boolean");
        return b;
    }
    const std::string& as_string(const std::string& what) const {
        if (kind != String) throw std::runtime_error("JSON: '" + what + "' must be a string");
        return str;
    }
};

class JsonParser {
public:
    explicit JsonParser(const std::string& text) : s_(text), i_(0) {}
    JsonValue parse() {
        JsonValue v = value();
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return v;
    }

private:
    const std::string& s_;
    size_t i_;

    [[noreturn]] void fail(const std::string& m) {
        throw std::runtime_error("JSON parse error at offset " + std::to_string(i_) + ": " + m);
    }
    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\r' || s_[i_] == '\t')) i_++;
    }
    bool lit(const char* w) {
        size_t n = 0;
        while (w[n]) n++;
        if (s_.compare(i_, n, w) == 0) { i_ += n; return true; }
        return false;
    }
    JsonValue value() {
        ws();
        if (i_ >= s_.size()) fail("unexpected end");
        char c = s_[i_];
        JsonValue v;
        if (c == '{') {
            v.kind = JsonValue::Object;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == '}') { i_++; return v; }
            for (;;) {
                ws();
                if (i_ >= s_.size() || s_[i_] != '"') fail("expected a string key");
                std::string k = string_lit();
                ws();
                if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':'");
                i_++;
                v.obj[k] = value();
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == '}') { i_++; break; }
                fail("expected ',' or '}'");
            }
        } else if (c == '[') {
            v.kind = JsonValue::Array;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == ']') { i_++; return v; }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == ']') { i_++; break; }
                fail("expected ',' or ']'");
            }
        } else if (c == '"') {
            v.kind = JsonValue::String;
            v.str = string_lit();
        } else if (lit("true")) {
            v.kind = JsonValue::Bool; v.b = true;
        } else if (lit("false")) {
            v.kind = JsonValue::Bool; v.b = false;
        } else if (lit("null")) {
            v.kind = JsonValue::Null;
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            size_t st = i_;
            bool integer = true;
            if (s_[i_] == '-') i_++;
            while (i_ < s_.size() && isdig(s_[i_])) i_++;
            if (i_ < s_.size() && s_[i_] == '.') { integer = false; i_++; while (i_ < s_.size() && isdig(s_[i_])) i_++; }
            if (i_ < s_.size() && (s_[i_] == 'e' || s_[i_] == 'E')) {
                integer = false;
                i_++;
                if (i_ < s_.size() && (s_[i_] == '+' || s_[i_] == '-')) i_++;
                while (i_ < s_.size() && isdig(s_[i_])) i_++;
            }
            std::string tok = s_.substr(st, i_ - st);
            char* end = nullptr;
            v.kind = JsonValue::Number;
            v.num = std::strtod(tok.c_str(), &end);
            if (!end || *end != '\0' || tok == "-") fail("bad number '" + tok + "'");
            v.is_integer = integer;
        } else {
            fail(std::string("unexpected character '") + c + "'");
        }
        return v;
    }
    static bool isdig(char c) { return c >= '0' && c <= '9'; }
    static void put_utf8(std::string& o, uint32_t cp) {
        if (cp < 0x80) o += (char)cp;
        else if (cp < 0x800) { o += (char)(0xC0 | (cp >> 6)); o += (char)(0x80 | (cp & 0x3F)); }
        else if (cp < 0x10000) { o += (char)(0xE0 | (cp >> 12)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F)); }
        else { o += (char)(0xF0 | (cp >> 18)); o += (char)(0x80 | ((cp >> 12) & 0x3F)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F)); }
    }
    uint32_t hex4() {
        if (i_ + 4 > s_.size()) fail("short \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; k++) {
            char c = s_[i_++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else fail("bad \\u escape");
        }
        return v;
    }
    std::string string_lit() {
        i_++;  // opening quote
        std::string o;
        while (i_ < s_.size()) {
            char c = s_[i_++];
            if (c == '"') return o;
            if (c != '\\') { o += c; continue; }
            if (i_ >= s_.size()) break;
            char e = s_[i_++];
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
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00 && i_ + 1 < s_.size() && s_[i_] == '\\' && s_[i_ + 1] == 'u') {
                        i_ += 2;
                        uint32_t lo = hex4();
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    put_utf8(o, cp);
                    break;
                }
                default: fail("bad escape");
            }
        }
        fail("unterminated string");
    }
};

}  // namespace cellsim
