#include "json.h"

#include <cctype>
#include <cmath>

#include "../../../include/c2g.h"

namespace c2g {
namespace {

struct Parser {
    const std::string& t;
    size_t p = 0;
    int line = 1;
    explicit Parser(const std::string& text) : t(text) {}

    [[noreturn]] void fail(const char* what) {
        throw JsonError(C2G_ERR_PARSE, std::string("json: ") + what + " at line " + std::to_string(line));
    }
    void ws() {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\r' || t[p] == '\n')) {
            if (t[p] == '\n') line++;
            p++;
        }
    }
    std::shared_ptr<Json> value() {
        ws();
        if (p >= t.size()) fail("unexpected end");
        char c = t[p];
        if (c == '{') return object();
        if (c == '[') return array();
        if (c == '"') { auto n = std::make_shared<Json>(); n->kind = Json::STRING; n->s = str(); return n; }
        if (c == '-' || std::isdigit((unsigned char)c)) return number();
        if (t.compare(p, 4, "true") == 0) { p += 4; auto n = std::make_shared<Json>(); n->kind = Json::BOOL; n->b = true; return n; }
        if (t.compare(p, 5, "false") == 0) { p += 5; auto n = std::make_shared<Json>(); n->kind = Json::BOOL; return n; }
        if (t.compare(p, 4, "null") == 0) { p += 4; return std::make_shared<Json>(); }
        fail("invalid value");
    }
    std::string str() {
        if (t[p] != '"') fail("expected '\"'");
        p++;
        std::string out;
        while (p < t.size() && t[p] != '"') {
            char c = t[p++];
            if (c == '\\') {
                if (p >= t.size()) break;
                char e = t[p++];
                switch (e) {
                    case '"': out.push_back('"'); break;
                    case '\\': out.push_back('\\'); break;
                    case '/': out.push_back('/'); break;
                    case 'b': out.push_back('\b'); break;
                    case 'f': out.push_back('\f'); break;
                    case 'n': out.push_back('\n'); break;
                    case 'r': out.push_back('\r'); break;
                    case 't': out.push_back('\t'); break;
                    default: out.push_back(e); break;
                }
            } else {
                if (c == '\n') line++;
                out.push_back(c);
            }
        }
        if (p >= t.size()) fail("unterminated string");
        p++;
        return out;
    }
    std::shared_ptr<Json> number() {
        bool neg = false;
        if (t[p] == '-') { neg = true; p++; }
        std::string ip, fp, ep;
        bool eneg = false;
        int stage = 0;
        while (p < t.size()) {
            char c = t[p];
            if (stage == 0) {
                if (std::isdigit((unsigned char)c)) ip.push_back(c);
                else if (c == '.') stage = 1;
                else if (std::tolower((unsigned char)c) == 'e') stage = 2;
                else break;
                p++;
            } else if (stage == 1) {
                if (std::isdigit((unsigned char)c)) fp.push_back(c);
                else if (c == '.') fail("invalid number");
                else if (std::tolower((unsigned char)c) == 'e') stage = 2;
                else break;
                p++;
            } else {
                if (stage == 2) {
                    if (c == '-') { eneg = true; p++; stage = 3; continue; }
                    if (c == '+') { p++; stage = 3; continue; }
                    stage = 3;
                }
                if (std::isdigit((unsigned char)c)) ep.push_back(c);
                else if (c == '.' || std::tolower((unsigned char)c) == 'e') fail("invalid number");
                else break;
                p++;
            }
        }
        if (ip.empty() && fp.empty() && ep.empty()) fail("invalid number");
        if (ip.size() > 1 && ip[0] == '0') fail("invalid number");
        auto n = std::make_shared<Json>();
        if (!ip.empty() && fp.empty() && ep.empty()) {
            long long v = 0;
            for (char c : ip) v = v * 10 + (c - '0');
            n->kind = Json::INT;
            n->i = neg ? -v : v;
            return n;
        }
        double v = 0;
        for (char c : ip) { v *= 10.0; v += c - '0'; }
        double tt = 10;
        for (char c : fp) { v += (c - '0') / tt; tt *= 10; }
        if (!ep.empty()) {
            long long e = 0;
            for (char c : ep) e = e * 10 + (c - '0');
            v *= std::pow(10.0, (double)(eneg ? -e : e));
        }
        n->kind = Json::FLOAT;
        n->f = neg ? -v : v;
        return n;
    }
    std::shared_ptr<Json> array() {
        p++;
        auto n = std::make_shared<Json>();
        n->kind = Json::ARRAY;
        ws();
        if (p < t.size() && t[p] == ']') { p++; return n; }
        while (true) {
            n->arr.push_back(value());
            ws();
            if (p >= t.size()) fail("unterminated array");
            if (t[p] == ',') { p++; continue; }
            if (t[p] == ']') { p++; return n; }
            fail("expected ',' or ']'");
        }
    }
    std::shared_ptr<Json> object() {
        p++;
        auto n = std::make_shared<Json>();
        n->kind = Json::OBJECT;
        ws();
        if (p < t.size() && t[p] == '}') { p++; return n; }
        while (true) {
            ws();
            if (p >= t.size()) fail("unterminated object");
            std::string k = str();
            ws();
            if (p >= t.size() || t[p] != ':') fail("expected ':'");
            p++;
            auto v = value();
            n->obj.insert({k, v});
            ws();
            if (p >= t.size()) fail("unterminated object");
            if (t[p] == ',') { p++; continue; }
            if (t[p] == '}') { p++; return n; }
            fail("expected ',' or '}'");
        }
    }
};

}  // namespace

std::shared_ptr<Json> Json::parse(const std::string& text) {
    Parser ps(text);
    auto v = ps.value();
    ps.ws();
    if (ps.p != text.size()) ps.fail("trailing characters");
    return v;
}

const Json& Json::at(const std::string& key) const {
    if (kind != OBJECT) throw JsonError(C2G_ERR_INVALID, "json: member '" + key + "' requested from a non-object");
    auto it = obj.find(key);
    if (it == obj.end()) throw JsonError(C2G_ERR_INVALID, "json: missing member '" + key + "'");
    return *it->second;
}

const Json& Json::at(size_t idx) const {
    if (kind != ARRAY || idx >= arr.size()) throw JsonError(C2G_ERR_INVALID, "json: array index out of range");
    return *arr[idx];
}

double Json::as_float() const {
    if (kind == FLOAT) return f;
    if (kind == INT) return (double)i;
    throw JsonError(C2G_ERR_INVALID, "json: expected a number");
}

long long Json::as_int() const {
    if (kind == INT) return i;
    if (kind == FLOAT) return (long long)f;
    throw JsonError(C2G_ERR_INVALID, "json: expected a number");
}

const std::string& Json::as_string() const {
    if (kind != STRING) throw JsonError(C2G_ERR_INVALID, "json: expected a string");
    return s;
}

}  // namespace c2g
