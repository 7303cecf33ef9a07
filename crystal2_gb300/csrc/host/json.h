// Minimal JSON reader for the reference's config and scene files.
//
// Numbers follow the reference parser's arithmetic (deps/TREngine/deps/SJson/SJson.cpp:81-231)
// rather than strtod: a literal without fraction or exponent is an integer node; otherwise the
// value is accumulated in double as int digits (v = v*10 + d), fraction digits (v += d / 10^k,
// with 10^k itself accumulated by repeated *10) and an exponent factor pow(10, e).  Scene floats
// are then narrowed to float, so using the same accumulation keeps every parsed parameter
// bit-identical to the reference's.  Duplicate object keys keep the first value (std::map::insert).
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace c2g {

struct JsonError : std::runtime_error {
    int code;  // C2G_ERR_PARSE or C2G_ERR_INVALID
    JsonError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

class Json {
public:
    enum Kind { NUL, BOOL, INT, FLOAT, STRING, ARRAY, OBJECT };
    Kind kind = NUL;
    bool b = false;
    long long i = 0;
    double f = 0.0;
    std::string s;
    std::vector<std::shared_ptr<Json>> arr;
    std::map<std::string, std::shared_ptr<Json>> obj;

    static std::shared_ptr<Json> parse(const std::string& text);

    bool has(const std::string& key) const { return kind == OBJECT && obj.count(key) != 0; }
    const Json& at(const std::string& key) const;     // throws JsonError(INVALID) when missing
    const Json& at(size_t idx) const;
    size_t size() const { return kind == ARRAY ? arr.size() : obj.size(); }
    double as_float() const;                            // GetFloat(): int nodes widen
    long long as_int() const;                           // GetInt(): float nodes truncate
    const std::string& as_string() const;
};

}  // namespace c2g
