// ORACLE (test infrastructure only) -- a project-owned subset of the
// nlohmann::json API, written from its documented behaviour, large enough to
// compile ibis's own sources unchanged.  Kept from nlohmann::json because ibis
// depends on it:
//   * objects keep their keys sorted (std::map), so items() and iteration
//     visit keys in lexicographic order (ibis numbers ghost cells in that order);
//   * an initializer list whose every element is a two-element array with a
//     string first builds an object, any other list builds an array;
//   * values convert implicitly to bool, numbers, std::string and (nested)
//     std::vector / std::map, and to nothing else; numbers convert between
//     integer and floating point with static_cast; at() throws on a missing
//     key or index;
//   * items() entries bind as [key, value] in a structured binding.
#ifndef IBIS_REF_SHIM_NLOHMANN_JSON_HPP
#define IBIS_REF_SHIM_NLOHMANN_JSON_HPP

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <istream>
#include <iterator>
#include <map>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {

class json;

namespace detail {
template <class T>
struct is_vector : std::false_type {};
template <class T, class A>
struct is_vector<std::vector<T, A>> : std::true_type {};
template <class T>
struct is_string_map : std::false_type {};
template <class T, class C, class A>
struct is_string_map<std::map<std::string, T, C, A>> : std::true_type {};
template <class T>
struct is_gettable
    : std::bool_constant<std::is_arithmetic_v<T> || std::is_same_v<T, std::string> || std::is_same_v<T, json>> {};
template <class T, class A>
struct is_gettable<std::vector<T, A>> : is_gettable<T> {};
template <class T, class C, class A>
struct is_gettable<std::map<std::string, T, C, A>> : is_gettable<T> {};
}  // namespace detail

class json {
public:
    enum class value_t { null, object, array, string, boolean, number_integer, number_unsigned, number_float };
    using object_t = std::map<std::string, json>;
    using array_t = std::vector<json>;
    using size_type = size_t;

    class exception : public std::runtime_error {
    public:
        using std::runtime_error::runtime_error;
    };
    class out_of_range : public exception {
    public:
        using exception::exception;
    };
    class type_error : public exception {
    public:
        using exception::exception;
    };
    class parse_error : public exception {
    public:
        using exception::exception;
    };

    // ------------------------------------------------------------ construction
    json() = default;
    json(std::nullptr_t) {}
    json(bool b) : t_(value_t::boolean), b_(b) {}
    template <class T, std::enable_if_t<std::is_integral_v<T> && !std::is_same_v<T, bool>, int> = 0>
    json(T v) {
        if (std::is_signed_v<T>) { t_ = value_t::number_integer; i_ = (int64_t)v; }
        else { t_ = value_t::number_unsigned; u_ = (uint64_t)v; }
    }
    template <class T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>
    json(T v) : t_(value_t::number_float), f_((double)v) {}
    json(const char* s) : t_(value_t::string), s_(s) {}
    json(const std::string& s) : t_(value_t::string), s_(s) {}
    template <class T>
    json(const std::vector<T>& v) : t_(value_t::array) {
        for (const auto& x : v) a_.push_back(json(x));
    }
    template <class T>
    json(const std::map<std::string, T>& m) : t_(value_t::object) {
        for (const auto& kv : m) o_[kv.first] = json(kv.second);
    }
    json(std::initializer_list<json> il) {
        bool obj = il.size() > 0;
        for (const json& e : il)
            if (!(e.t_ == value_t::array && e.a_.size() == 2 && e.a_[0].t_ == value_t::string)) obj = false;
        if (obj) {
            t_ = value_t::object;
            for (const json& e : il) o_[e.a_[0].s_] = e.a_[1];
        } else {
            t_ = value_t::array;
            a_.assign(il.begin(), il.end());
        }
    }
    json(const json&) = default;
    json(json&&) = default;
    json& operator=(const json&) = default;
    json& operator=(json&&) = default;

    static json array() { json j; j.t_ = value_t::array; return j; }
    static json array(std::initializer_list<json> il) { json j; j.t_ = value_t::array; j.a_.assign(il.begin(), il.end()); return j; }
    static json object() { json j; j.t_ = value_t::object; return j; }

    // ------------------------------------------------------------ parsing
    static json parse(std::istream& in) {
        std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        return parse(text);
    }
    static json parse(const std::string& text) {
        size_t p = 0;
        json j = parse_value(text, p);
        skip_ws(text, p);
        if (p != text.size()) throw parse_error("json::parse: trailing characters");
        return j;
    }
    static json parse(const char* text) { return parse(std::string(text)); }

    // ------------------------------------------------------------ inspection
    value_t type() const { return t_; }
    bool is_null() const { return t_ == value_t::null; }
    bool is_object() const { return t_ == value_t::object; }
    bool is_array() const { return t_ == value_t::array; }
    bool is_string() const { return t_ == value_t::string; }
    bool is_boolean() const { return t_ == value_t::boolean; }
    bool is_number() const { return is_number_integer() || t_ == value_t::number_float; }
    bool is_number_integer() const { return t_ == value_t::number_integer || t_ == value_t::number_unsigned; }
    bool is_number_unsigned() const { return t_ == value_t::number_unsigned; }
    bool is_number_float() const { return t_ == value_t::number_float; }
    bool is_primitive() const { return !is_object() && !is_array(); }
    bool is_structured() const { return is_object() || is_array(); }

    size_t size() const {
        if (t_ == value_t::object) return o_.size();
        if (t_ == value_t::array) return a_.size();
        return t_ == value_t::null ? 0 : 1;
    }
    bool empty() const { return size() == 0; }

    // ------------------------------------------------------------ element access
    json& at(const std::string& k) {
        if (t_ != value_t::object) throw type_error("json::at(\"" + k + "\") on a non-object");
        auto it = o_.find(k);
        if (it == o_.end()) throw out_of_range("json::at: key '" + k + "' not found");
        return it->second;
    }
    const json& at(const std::string& k) const { return const_cast<json*>(this)->at(k); }
    json& at(size_t i) {
        if (t_ != value_t::array) throw type_error("json::at(index) on a non-array");
        if (i >= a_.size()) throw out_of_range("json::at: index out of range");
        return a_[i];
    }
    const json& at(size_t i) const { return const_cast<json*>(this)->at(i); }
    json& operator[](const std::string& k) {
        if (t_ == value_t::null) t_ = value_t::object;
        if (t_ != value_t::object) throw type_error("json::operator[](\"" + k + "\") on a non-object");
        return o_[k];
    }
    json& operator[](const char* k) { return (*this)[std::string(k)]; }
    const json& operator[](const std::string& k) const { return at(k); }
    const json& operator[](const char* k) const { return at(std::string(k)); }
    template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
    json& operator[](I i) {
        if (t_ == value_t::null) t_ = value_t::array;
        if (t_ != value_t::array) throw type_error("json::operator[](index) on a non-array");
        if ((size_t)i >= a_.size()) a_.resize((size_t)i + 1);
        return a_[(size_t)i];
    }
    template <class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
    const json& operator[](I i) const { return at((size_t)i); }
    bool contains(const std::string& k) const { return t_ == value_t::object && o_.count(k) != 0; }
    size_t count(const std::string& k) const { return contains(k) ? 1 : 0; }
    template <class T>
    T value(const std::string& k, const T& def) const {
        return contains(k) ? at(k).get<T>() : def;
    }
    std::string value(const std::string& k, const char* def) const {
        return contains(k) ? at(k).get<std::string>() : std::string(def);
    }

    void push_back(const json& v) {
        if (t_ == value_t::null) t_ = value_t::array;
        if (t_ != value_t::array) throw type_error("json::push_back on a non-array");
        a_.push_back(v);
    }
    template <class... A>
    json& emplace_back(A&&... a) {
        push_back(json(std::forward<A>(a)...));
        return a_.back();
    }
    void clear() { a_.clear(); o_.clear(); s_.clear(); }
    size_t erase(const std::string& k) { return o_.erase(k); }

    // ------------------------------------------------------------ iteration
    template <bool C>
    class iter {
        using J = std::conditional_t<C, const json, json>;
        using AI = std::conditional_t<C, array_t::const_iterator, array_t::iterator>;
        using OI = std::conditional_t<C, object_t::const_iterator, object_t::iterator>;

    public:
        using iterator_category = std::forward_iterator_tag;
        using value_type = json;
        using difference_type = std::ptrdiff_t;
        using pointer = J*;
        using reference = J&;
        iter() = default;
        iter(J* owner, AI a) : owner_(owner), kind_(1), a_(a) {}
        iter(J* owner, OI o) : owner_(owner), kind_(2), o_(o) {}
        iter(J* owner, bool end) : owner_(owner), kind_(0), end_(end) {}
        J& operator*() const { return kind_ == 1 ? *a_ : (kind_ == 2 ? o_->second : *owner_); }
        J* operator->() const { return &**this; }
        iter& operator++() {
            if (kind_ == 1) ++a_;
            else if (kind_ == 2) ++o_;
            else end_ = true;
            return *this;
        }
        iter operator++(int) { iter t = *this; ++*this; return t; }
        bool operator==(const iter& x) const {
            if (kind_ != x.kind_) return false;
            return kind_ == 1 ? a_ == x.a_ : (kind_ == 2 ? o_ == x.o_ : end_ == x.end_);
        }
        bool operator!=(const iter& x) const { return !(*this == x); }
        std::string key() const {
            if (kind_ != 2) throw type_error("json iterator: key() of a non-object");
            return o_->first;
        }
        J& value() const { return **this; }

    private:
        J* owner_ = nullptr;
        int kind_ = 0;  // 0 primitive, 1 array, 2 object
        AI a_{};
        OI o_{};
        bool end_ = false;
    };
    using iterator = iter<false>;
    using const_iterator = iter<true>;
    iterator begin() {
        if (t_ == value_t::array) return iterator(this, a_.begin());
        if (t_ == value_t::object) return iterator(this, o_.begin());
        return iterator(this, t_ == value_t::null);
    }
    iterator end() {
        if (t_ == value_t::array) return iterator(this, a_.end());
        if (t_ == value_t::object) return iterator(this, o_.end());
        return iterator(this, true);
    }
    const_iterator begin() const {
        if (t_ == value_t::array) return const_iterator(this, a_.cbegin());
        if (t_ == value_t::object) return const_iterator(this, o_.cbegin());
        return const_iterator(this, t_ == value_t::null);
    }
    const_iterator end() const {
        if (t_ == value_t::array) return const_iterator(this, a_.cend());
        if (t_ == value_t::object) return const_iterator(this, o_.cend());
        return const_iterator(this, true);
    }
    const_iterator cbegin() const { return begin(); }
    const_iterator cend() const { return end(); }
    iterator find(const std::string& k) {
        return t_ == value_t::object ? iterator(this, o_.find(k)) : end();
    }
    const_iterator find(const std::string& k) const {
        return t_ == value_t::object ? const_iterator(this, o_.find(k)) : end();
    }

    // key/value pairs: object keys in sorted order, array indices as strings;
    // also tuple-like (for (auto& [key, value] : j.items()))
    struct item {
        std::string k;
        json* v;
        const std::string& key() const { return k; }
        json& value() const { return *v; }
        template <size_t N>
        decltype(auto) get() const {
            if constexpr (N == 0) return (k);
            else return (*v);
        }
    };
    struct const_item {
        std::string k;
        const json* v;
        const std::string& key() const { return k; }
        const json& value() const { return *v; }
        template <size_t N>
        decltype(auto) get() const {
            if constexpr (N == 0) return (k);
            else return (*v);
        }
    };
    std::vector<item> items() {
        std::vector<item> r;
        if (t_ == value_t::object)
            for (auto& kv : o_) r.push_back({kv.first, &kv.second});
        else if (t_ == value_t::array)
            for (size_t i = 0; i < a_.size(); i++) r.push_back({std::to_string(i), &a_[i]});
        return r;
    }
    std::vector<const_item> items() const {
        std::vector<const_item> r;
        if (t_ == value_t::object)
            for (const auto& kv : o_) r.push_back({kv.first, &kv.second});
        else if (t_ == value_t::array)
            for (size_t i = 0; i < a_.size(); i++) r.push_back({std::to_string(i), &a_[i]});
        return r;
    }

    // ------------------------------------------------------------ conversion
    template <class T>
    T get() const {
        using U = std::remove_cv_t<std::remove_reference_t<T>>;
        if constexpr (std::is_same_v<U, json>) {
            return *this;
        } else if constexpr (std::is_same_v<U, bool>) {
            if (t_ != value_t::boolean) throw type_error("json: value is not a boolean");
            return b_;
        } else if constexpr (std::is_arithmetic_v<U>) {
            switch (t_) {
                case value_t::number_integer: return static_cast<U>(i_);
                case value_t::number_unsigned: return static_cast<U>(u_);
                case value_t::number_float: return static_cast<U>(f_);
                case value_t::boolean: return static_cast<U>(b_);
                default: throw type_error("json: value is not a number");
            }
        } else if constexpr (std::is_same_v<U, std::string>) {
            if (t_ != value_t::string) throw type_error("json: value is not a string");
            return s_;
        } else if constexpr (detail::is_vector<U>::value) {
            if (t_ != value_t::array) throw type_error("json: value is not an array");
            U out;
            for (const json& e : a_) out.push_back(e.get<typename U::value_type>());
            return out;
        } else if constexpr (detail::is_string_map<U>::value) {
            if (t_ != value_t::object) throw type_error("json: value is not an object");
            U out;
            for (const auto& kv : o_) out[kv.first] = kv.second.get<typename U::mapped_type>();
            return out;
        } else {
            static_assert(sizeof(U) == 0, "json::get: unsupported type");
        }
    }
    template <class T>
    void get_to(T& v) const { v = get<T>(); }
    template <class T, std::enable_if_t<detail::is_gettable<T>::value && !std::is_same_v<T, char>, int> = 0>
    operator T() const {
        return get<T>();
    }

    // ------------------------------------------------------------ comparison
    friend bool operator==(const json& a, const json& b) {
        if (a.is_number() && b.is_number()) {
            if (a.t_ == value_t::number_float || b.t_ == value_t::number_float)
                return a.get<double>() == b.get<double>();
            if (a.t_ == value_t::number_unsigned && b.t_ == value_t::number_unsigned) return a.u_ == b.u_;
            return a.get<int64_t>() == b.get<int64_t>();
        }
        if (a.t_ != b.t_) return false;
        switch (a.t_) {
            case value_t::null: return true;
            case value_t::boolean: return a.b_ == b.b_;
            case value_t::string: return a.s_ == b.s_;
            case value_t::array: return a.a_ == b.a_;
            case value_t::object: return a.o_ == b.o_;
            default: return false;
        }
    }
    friend bool operator!=(const json& a, const json& b) { return !(a == b); }
    friend bool operator==(const json& a, const char* s) { return a == json(s); }
    friend bool operator==(const char* s, const json& a) { return a == json(s); }
    friend bool operator!=(const json& a, const char* s) { return !(a == json(s)); }
    friend bool operator!=(const char* s, const json& a) { return !(a == json(s)); }
    friend bool operator==(const json& a, const std::string& s) { return a == json(s); }
    friend bool operator==(const std::string& s, const json& a) { return a == json(s); }
    friend bool operator!=(const json& a, const std::string& s) { return !(a == json(s)); }
    friend bool operator!=(const std::string& s, const json& a) { return !(a == json(s)); }
    template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
    friend bool operator==(const json& a, T v) { return a == json(v); }
    template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
    friend bool operator==(T v, const json& a) { return a == json(v); }
    template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
    friend bool operator!=(const json& a, T v) { return !(a == json(v)); }
    template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
    friend bool operator!=(T v, const json& a) { return !(a == json(v)); }

    // ------------------------------------------------------------ serialisation
    std::string dump(int indent = -1) const {
        std::string out;
        write(out, indent, 0);
        return out;
    }
    friend std::ostream& operator<<(std::ostream& os, const json& j) { return os << j.dump(); }
    friend std::istream& operator>>(std::istream& is, json& j) {
        j = parse(is);
        return is;
    }

private:
    static std::string num_to_string(double x) {
        if (!std::isfinite(x)) return "null";
        char buf[40];
        for (int prec = 15; prec <= 17; prec++) {  // the shortest of these that reads back exactly
            std::snprintf(buf, sizeof buf, "%.*g", prec, x);
            if (std::strtod(buf, nullptr) == x) break;
        }
        std::string s(buf);
        if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
        return s;
    }
    static void write_string(std::string& out, const std::string& s) {
        out += '"';
        for (char c : s) {
            switch (c) {
                case '"': out += "\\\""; break;
                case '\\': out += "\\\\"; break;
                case '\n': out += "\\n"; break;
                case '\t': out += "\\t"; break;
                case '\r': out += "\\r"; break;
                case '\b': out += "\\b"; break;
                case '\f': out += "\\f"; break;
                default:
                    if ((unsigned char)c < 0x20) {
                        char b[8];
                        std::snprintf(b, sizeof b, "\\u%04x", (unsigned)(unsigned char)c);
                        out += b;
                    } else {
                        out += c;
                    }
            }
        }
        out += '"';
    }
    void write(std::string& out, int indent, int level) const {
        const bool pretty = indent >= 0;
        auto nl = [&](int lv) {
            if (pretty) { out += '\n'; out.append((size_t)(indent * lv), ' '); }
        };
        switch (t_) {
            case value_t::null: out += "null"; break;
            case value_t::boolean: out += b_ ? "true" : "false"; break;
            case value_t::number_integer: out += std::to_string(i_); break;
            case value_t::number_unsigned: out += std::to_string(u_); break;
            case value_t::number_float: out += num_to_string(f_); break;
            case value_t::string: write_string(out, s_); break;
            case value_t::array: {
                if (a_.empty()) { out += "[]"; break; }
                out += '[';
                for (size_t i = 0; i < a_.size(); i++) {
                    if (i) out += ',';
                    nl(level + 1);
                    a_[i].write(out, indent, level + 1);
                }
                nl(level);
                out += ']';
                break;
            }
            case value_t::object: {
                if (o_.empty()) { out += "{}"; break; }
                out += '{';
                bool first = true;
                for (const auto& kv : o_) {
                    if (!first) out += ',';
                    first = false;
                    nl(level + 1);
                    write_string(out, kv.first);
                    out += pretty ? ": " : ":";
                    kv.second.write(out, indent, level + 1);
                }
                nl(level);
                out += '}';
                break;
            }
        }
    }

    static void skip_ws(const std::string& t, size_t& p) {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\n' || t[p] == '\r' || t[p] == '\t')) p++;
    }
    static std::string parse_string(const std::string& t, size_t& p) {
        if (t[p] != '"') throw parse_error("json::parse: expected a string");
        p++;
        std::string s;
        while (p < t.size() && t[p] != '"') {
            char c = t[p++];
            if (c != '\\') { s += c; continue; }
            if (p >= t.size()) break;
            char e = t[p++];
            switch (e) {
                case 'n': s += '\n'; break;
                case 't': s += '\t'; break;
                case 'r': s += '\r'; break;
                case 'b': s += '\b'; break;
                case 'f': s += '\f'; break;
                case 'u': {
                    unsigned cp = (unsigned)std::strtoul(t.substr(p, 4).c_str(), nullptr, 16);
                    p += 4;
                    if (cp < 0x80) s += (char)cp;
                    else if (cp < 0x800) { s += (char)(0xC0 | (cp >> 6)); s += (char)(0x80 | (cp & 0x3F)); }
                    else { s += (char)(0xE0 | (cp >> 12)); s += (char)(0x80 | ((cp >> 6) & 0x3F)); s += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: s += e;
            }
        }
        if (p >= t.size()) throw parse_error("json::parse: unterminated string");
        p++;
        return s;
    }
    static json parse_value(const std::string& t, size_t& p) {
        skip_ws(t, p);
        if (p >= t.size()) throw parse_error("json::parse: unexpected end of input");
        const char c = t[p];
        if (c == '{') {
            json j = object();
            p++;
            skip_ws(t, p);
            if (p < t.size() && t[p] == '}') { p++; return j; }
            while (true) {
                skip_ws(t, p);
                std::string k = parse_string(t, p);
                skip_ws(t, p);
                if (p >= t.size() || t[p] != ':') throw parse_error("json::parse: expected ':'");
                p++;
                j.o_[k] = parse_value(t, p);
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',') { p++; continue; }
                if (p < t.size() && t[p] == '}') { p++; return j; }
                throw parse_error("json::parse: expected ',' or '}'");
            }
        }
        if (c == '[') {
            json j = array();
            p++;
            skip_ws(t, p);
            if (p < t.size() && t[p] == ']') { p++; return j; }
            while (true) {
                j.a_.push_back(parse_value(t, p));
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',') { p++; continue; }
                if (p < t.size() && t[p] == ']') { p++; return j; }
                throw parse_error("json::parse: expected ',' or ']'");
            }
        }
        if (c == '"') return json(parse_string(t, p));
        if (t.compare(p, 4, "true") == 0) { p += 4; return json(true); }
        if (t.compare(p, 5, "false") == 0) { p += 5; return json(false); }
        if (t.compare(p, 4, "null") == 0) { p += 4; return json(); }
        size_t q = p;
        bool flt = false;
        if (q < t.size() && (t[q] == '-' || t[q] == '+')) q++;
        while (q < t.size() && (std::isdigit((unsigned char)t[q]) || t[q] == '.' || t[q] == 'e' || t[q] == 'E' ||
                                t[q] == '-' || t[q] == '+')) {
            if (t[q] == '.' || t[q] == 'e' || t[q] == 'E') flt = true;
            q++;
        }
        if (q == p) throw parse_error("json::parse: unexpected character");
        const std::string num = t.substr(p, q - p);
        p = q;
        if (flt) return json(std::strtod(num.c_str(), nullptr));
        if (num[0] == '-') return json((int64_t)std::strtoll(num.c_str(), nullptr, 10));
        return json((uint64_t)std::strtoull(num.c_str(), nullptr, 10));
    }

    value_t t_ = value_t::null;
    bool b_ = false;
    int64_t i_ = 0;
    uint64_t u_ = 0;
    double f_ = 0.0;
    std::string s_;
    array_t a_;
    object_t o_;
};

}  // namespace nlohmann

namespace std {
template <>
struct tuple_size<nlohmann::json::item> : std::integral_constant<size_t, 2> {};
template <>
struct tuple_element<0, nlohmann::json::item> {
    using type = const std::string;
};
template <>
struct tuple_element<1, nlohmann::json::item> {
    using type = nlohmann::json;
};
template <>
struct tuple_size<nlohmann::json::const_item> : std::integral_constant<size_t, 2> {};
template <>
struct tuple_element<0, nlohmann::json::const_item> {
    using type = const std::string;
};
template <>
struct tuple_element<1, nlohmann::json::const_item> {
    using type = const nlohmann::json;
};
}  // namespace std

#endif
