// sc_json.hpp -- a small JSON reader for the setup surface of the step
// (config.json and the universe-config/gen/*.json tables).  The reference
// reads these with jsoncpp (config.cuh:46-64, chemistry.cuh:10-33,
// interactions.cuh:17-54); this reader keeps the distinctions its loaders rely
// on: integer vs real literals, explicit null, and numbers parsed to double
// first (a float field is the double value rounded to float, as jsoncpp's
// asFloat() does).
#pragma once

#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace scjson {

struct Value {
    enum Type { Null, Bool, Int, Real, String, Array, Object };
    Type type = Null;
    bool b = false;
    long long i = 0;
    double d = 0.0;
    std::string s;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;

    const Value *find(const char *key) const {
        if (type != Object) return nullptr;
        for (const auto &kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    size_t size() const { return type == Array ? arr.size() : type == Object ? obj.size() : 0; }
    bool is_number() const { return type == Int || type == Real; }
    double as_double() const { return type == Int ? (double)i : type == Real ? d : type == Bool ? (b ? 1.0 : 0.0) : 0.0; }
};

class Parser {
  public:
    Parser(const char *text, size_t n) : p_(text), end_(text + n) {}
    bool parse(Value &out, std::string &err) {
        skip();
        if (!value(out)) { err = err_.empty() ? "malformed JSON" : err_; return false; }
        skip();
        if (p_ != end_) { err = "trailing characters after JSON value"; return false; }
        return true;
    }

  private:
    const char *p_, *end_;
    std::string err_;
    int depth_ = 0;

    void skip() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) p_++;
    }
    bool lit(const char *w) {
        size_t n = strlen(w);
        if ((size_t)(end_ - p_) < n || memcmp(p_, w, n) != 0) return false;
        p_ += n;
        return true;
    }
    bool value(Value &v) {
        if (p_ >= end_) { err_ = "unexpected end of JSON"; return false; }
        if (++depth_ > 256) { err_ = "JSON nested too deeply"; return false; }
        bool ok = false;
        char c = *p_;
        if (c == '{') ok = object(v);
        else if (c == '[') ok = array(v);
        else if (c == '"') { v.type = Value::String; ok = string(v.s); }
        else if (c == 't') { ok = lit("true"); v.type = Value::Bool; v.b = true; }
        else if (c == 'f') { ok = lit("false"); v.type = Value::Bool; v.b = false; }
        else if (c == 'n') { ok = lit("null"); v.type = Value::Null; }
        else ok = number(v);
        depth_--;
        return ok;
    }
    bool number(Value &v) {
        const char *s = p_;
        if (p_ < end_ && (*p_ == '-' || *p_ == '+')) p_++;
        bool real = false, digits = false;
        while (p_ < end_) {
            char c = *p_;
            if (c >= '0' && c <= '9') { digits = true; p_++; }
            else if (c == '.' || c == 'e' || c == 'E') { real = true; p_++; }
            else if ((c == '-' || c == '+') && (p_[-1] == 'e' || p_[-1] == 'E')) p_++;
            else break;
        }
        if (!digits) { err_ = "invalid JSON value"; return false; }
        std::string t(s, p_);
        char *e = nullptr;
        if (!real) {
            long long iv = strtoll(t.c_str(), &e, 10);
            if (e && *e == '\0') { v.type = Value::Int; v.i = iv; return true; }
        }
        double dv = strtod(t.c_str(), &e);
        if (!e || *e != '\0') { err_ = "invalid JSON number"; return false; }
        v.type = Value::Real;
        v.d = dv;
        return true;
    }
    bool string(std::string &out) {
        p_++;  // opening quote
        out.clear();
        while (p_ < end_ && *p_ != '"') {
            char c = *p_++;
            if (c == '\\') {
                if (p_ >= end_) break;
                char e = *p_++;
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (end_ - p_ < 4) { err_ = "bad \\u escape"; return false; }
                        unsigned cp = (unsigned)strtoul(std::string(p_, p_ + 4).c_str(), nullptr, 16);
                        p_ += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (p_ >= end_) { err_ = "unterminated JSON string"; return false; }
        p_++;
        return true;
    }
    bool array(Value &v) {
        v.type = Value::Array;
        p_++;
        skip();
        if (p_ < end_ && *p_ == ']') { p_++; return true; }
        while (true) {
            skip();
            v.arr.emplace_back();
            if (!value(v.arr.back())) return false;
            skip();
            if (p_ < end_ && *p_ == ',') { p_++; continue; }
            if (p_ < end_ && *p_ == ']') { p_++; return true; }
            err_ = "expected , or ] in JSON array";
            return false;
        }
    }
    bool object(Value &v) {
        v.type = Value::Object;
        p_++;
        skip();
        if (p_ < end_ && *p_ == '}') { p_++; return true; }
        while (true) {
            skip();
            if (p_ >= end_ || *p_ != '"') { err_ = "expected key in JSON object"; return false; }
            std::string key;
            if (!string(key)) return false;
            skip();
            if (p_ >= end_ || *p_ != ':') { err_ = "expected : in JSON object"; return false; }
            p_++;
            skip();
            v.obj.emplace_back(key, Value());
            if (!value(v.obj.back().second)) return false;
            skip();
            if (p_ < end_ && *p_ == ',') { p_++; continue; }
            if (p_ < end_ && *p_ == '}') { p_++; return true; }
            err_ = "expected , or } in JSON object";
            return false;
        }
    }
};

inline bool parse(const std::string &text, Value &out, std::string &err) {
    Parser ps(text.data(), text.size());
    return ps.parse(out, err);
}

}  // namespace scjson
