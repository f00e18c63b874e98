// Host stand-in for jsoncpp's <json/json.h> (oracle only): the subset of
// Json::Value the reference's loaders call (config.cuh:46-64,
// chemistry.cuh:10-33, interactions.cuh:17-54, 148-181), with jsoncpp's
// conversion rules -- asInt() of null is 0, get(key, default) returns the
// member even when it is an explicit null, asFloat() rounds the double value.
#pragma once
#include <istream>
#include <iterator>
#include <stdexcept>
#include <string>
#include "sc_json.hpp"

namespace Json {

class Value {
  public:
    Value() {}
    Value(int v) { v_.type = scjson::Value::Int; v_.i = v; }
    Value(bool v) { v_.type = scjson::Value::Bool; v_.b = v; }
    Value(double v) { v_.type = scjson::Value::Real; v_.d = v; }
    explicit Value(const scjson::Value &v) : v_(v) {}

    unsigned size() const { return (unsigned)v_.size(); }
    bool isNull() const { return v_.type == scjson::Value::Null; }
    Value operator[](int i) const {
        if (v_.type != scjson::Value::Array || i < 0 || (size_t)i >= v_.arr.size()) return Value();
        return Value(v_.arr[(size_t)i]);
    }
    Value operator[](unsigned i) const { return (*this)[(int)i]; }
    Value operator[](const char *key) const {
        const scjson::Value *m = v_.find(key);
        return m ? Value(*m) : Value();
    }
    Value operator[](const std::string &key) const { return (*this)[key.c_str()]; }
    Value get(const char *key, const Value &def) const {
        const scjson::Value *m = v_.find(key);
        return m ? Value(*m) : def;
    }
    int asInt() const {
        switch (v_.type) {
            case scjson::Value::Null: return 0;
            case scjson::Value::Bool: return v_.b ? 1 : 0;
            case scjson::Value::Int: return (int)v_.i;
            case scjson::Value::Real: return (int)v_.d;
            default: throw std::runtime_error("Value is not convertible to Int.");
        }
    }
    float asFloat() const {
        switch (v_.type) {
            case scjson::Value::Null: return 0.0f;
            case scjson::Value::Bool: return v_.b ? 1.0f : 0.0f;
            case scjson::Value::Int: return (float)v_.i;
            case scjson::Value::Real: return (float)v_.d;
            default: throw std::runtime_error("Value is not convertible to float.");
        }
    }
    double asDouble() const { return v_.as_double(); }
    bool asBool() const {
        switch (v_.type) {
            case scjson::Value::Null: return false;
            case scjson::Value::Bool: return v_.b;
            case scjson::Value::Int: return v_.i != 0;
            case scjson::Value::Real: return v_.d != 0.0;
            default: throw std::runtime_error("Value is not convertible to bool.");
        }
    }
    const char *asCString() const { return v_.s.c_str(); }
    std::string asString() const { return v_.s; }

  private:
    scjson::Value v_;
};

inline std::istream &operator>>(std::istream &in, Value &v) {
    std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    scjson::Value root;
    std::string err;
    if (!scjson::parse(text, root, err)) throw std::runtime_error(err);
    v = Value(root);
    return in;
}

}  // namespace Json
