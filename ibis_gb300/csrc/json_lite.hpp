// Minimal JSON reader for ibis's config/config.json.
//
// Objects keep their keys in a std::map, so iteration is in lexicographic key
// order. ibis reads its config with nlohmann::json, whose default object type
// is also an ordered std::map; the order matters because ghost-cell ids are
// handed out while iterating `grid.boundaries` (reference: src/grid/grid/grid.h:414).
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ibisgb {

class Json {
public:
    enum class Kind { Null, Bool, Number, String, Array, Object };

    Json() = default;
    static Json number(double v) { Json j; j.kind_ = Kind::Number; j.num_ = v; return j; }
    static Json boolean(bool v) { Json j; j.kind_ = Kind::Bool; j.b_ = v; return j; }
    static Json string(std::string s) { Json j; j.kind_ = Kind::String; j.str_ = std::move(s); return j; }

    static Json parse(const std::string& text) {
        size_t pos = 0;
        Json j = parse_value(text, pos);
        skip_ws(text, pos);
        if (pos != text.size()) throw std::runtime_error("json: trailing characters");
        return j;
    }

    Kind kind() const { return kind_; }
    bool is_object() const { return kind_ == Kind::Object; }
    bool is_array() const { return kind_ == Kind::Array; }
    bool is_number() const { return kind_ == Kind::Number; }
    bool is_string() const { return kind_ == Kind::String; }
    bool is_bool() const { return kind_ == Kind::Bool; }

    bool contains(const std::string& key) const {
        return kind_ == Kind::Object && obj_.count(key) != 0;
    }
    const Json& at(const std::string& key) const {
        if (kind_ != Kind::Object) throw std::runtime_error("json: '" + key + "' looked up in a non-object");
        auto it = obj_.find(key);
        if (it == obj_.end()) throw std::runtime_error("json: missing key '" + key + "'");
        return it->second;
    }
    const Json& at(size_t i) const {
        if (kind_ != Kind::Array || i >= arr_.size()) throw std::runtime_error("json: bad array index");
        return arr_[i];
    }
    size_t size() const { return kind_ == Kind::Array ? arr_.size() : obj_.size(); }
    const std::map<std::string, Json>& items() const { return obj_; }
    const std::vector<Json>& elements() const { return arr_; }

    double as_double() const {
        if (kind_ == Kind::Number) return num_;
        if (kind_ == Kind::Bool) return b_ ? 1.0 : 0.0;
        throw std::runtime_error("json: value is not a number");
    }
    long long as_int() const { return (long long)as_double(); }
    bool as_bool() const {
        if (kind_ == Kind::Bool) return b_;
        if (kind_ == Kind::Number) return num_ != 0.0;
        throw std::runtime_error("json: value is not a bool");
    }
    const std::string& as_string() const {
        if (kind_ != Kind::String) throw std::runtime_error("json: value is not a string");
        return str_;
    }
    std::vector<double> as_doubles() const {
        std::vector<double> out;
        for (const auto& e : elements()) out.push_back(e.as_double());
        return out;
    }

    // typed lookups with defaults, for the few build-only keys
    double get(const std::string& key, double dflt) const {
        return contains(key) ? at(key).as_double() : dflt;
    }
    std::string get(const std::string& key, const std::string& dflt) const {
        return contains(key) ? at(key).as_string() : dflt;
    }

private:
    Kind kind_ = Kind::Null;
    bool b_ = false;
    double num_ = 0.0;
    std::string str_;
    std::vector<Json> arr_;
    std::map<std::string, Json> obj_;

    static void skip_ws(const std::string& s, size_t& p) {
        while (p < s.size() && (s[p] == ' ' || s[p] == '\n' || s[p] == '\t' || s[p] == '\r')) p++;
    }
    static void expect(const std::string& s, size_t& p, char c) {
        skip_ws(s, p);
        if (p >= s.size() || s[p] != c) throw std::runtime_error(std::string("json: expected '") + c + "'");
        p++;
    }
    static std::string parse_string(const std::string& s, size_t& p) {
        expect(s, p, '"');
        std::string out;
        while (p < s.size() && s[p] != '"') {
            char c = s[p++];
            if (c == '\\') {
                if (p >= s.size()) break;
                char e = s[p++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {  // keep ASCII code points, replace the rest
                        unsigned code = (unsigned)std::strtoul(s.substr(p, 4).c_str(), nullptr, 16);
                        p += 4;
                        out += code < 128 ? (char)code : '?';
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (p >= s.size()) throw std::runtime_error("json: unterminated string");
        p++;
        return out;
    }
    static Json parse_value(const std::string& s, size_t& p) {
        skip_ws(s, p);
        if (p >= s.size()) throw std::runtime_error("json: unexpected end");
        char c = s[p];
        if (c == '{') {
            Json j; j.kind_ = Kind::Object; p++;
            skip_ws(s, p);
            if (p < s.size() && s[p] == '}') { p++; return j; }
            while (true) {
                std::string key = parse_string(s, p);
                expect(s, p, ':');
                j.obj_[key] = parse_value(s, p);
                skip_ws(s, p);
                if (p < s.size() && s[p] == ',') { p++; continue; }
                expect(s, p, '}');
                return j;
            }
        }
        if (c == '[') {
            Json j; j.kind_ = Kind::Array; p++;
            skip_ws(s, p);
            if (p < s.size() && s[p] == ']') { p++; return j; }
            while (true) {
                j.arr_.push_back(parse_value(s, p));
                skip_ws(s, p);
                if (p < s.size() && s[p] == ',') { p++; continue; }
                expect(s, p, ']');
                return j;
            }
        }
        if (c == '"') return string(parse_string(s, p));
        if (s.compare(p, 4, "true") == 0) { p += 4; return boolean(true); }
        if (s.compare(p, 5, "false") == 0) { p += 5; return boolean(false); }
        if (s.compare(p, 4, "null") == 0) { p += 4; return Json(); }
        if (s.compare(p, 8, "Infinity") == 0) { p += 8; return number(1e308 * 10); }
        if (s.compare(p, 9, "-Infinity") == 0) { p += 9; return number(-1e308 * 10); }
        if (s.compare(p, 3, "NaN") == 0) { p += 3; return number(0.0 / 0.0 * 0.0 + __builtin_nan("")); }
        const char* begin = s.c_str() + p;
        char* end = nullptr;
        double v = std::strtod(begin, &end);
        if (end == begin) throw std::runtime_error("json: bad value");
        p += (size_t)(end - begin);
        return number(v);
    }
};

inline std::string read_text_file(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open " + path);
    std::string out;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
    std::fclose(f);
    return out;
}

}  // namespace ibisgb
