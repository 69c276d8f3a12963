#include "props.h"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <sstream>

namespace sg {

int Props::get_int(const std::string& k, int def) const {
    if (!has(k)) return def;
    try {
        return std::stoi(get(k));
    } catch (...) {
        throw SgError("Could not convert property \"" + k + "\" (" + get(k) + ") to integer!");
    }
}

float Props::get_float(const std::string& k, float def) const {
    if (!has(k)) return def;
    try {
        return std::stof(get(k));
    } catch (...) {
        throw SgError("Could not convert property \"" + k + "\" (" + get(k) + ") to float!");
    }
}

Props* Props::set(const std::string& k, const std::string& v) {
    if (!props_.count(k)) keys_.push_back(k);
    props_[k] = v;
    return this;
}

Props* Props::set_child(const std::string& k, const Props& c) {
    if (!children_.count(k)) child_keys_.push_back(k);
    children_[k].reset(new Props(c));
    return this;
}

Props* Props::add_to_array(const std::string& k, const std::string& v) {
    if (!arrays_.count(k)) array_keys_.push_back(k);
    arrays_[k].push_back(v);
    return this;
}

std::vector<Props*> Props::child_array(const std::string& k) const {
    std::vector<Props*> out;
    auto it = child_arrays_.find(k);
    if (it != child_arrays_.end())
        for (auto& p : it->second) out.push_back(p.get());
    return out;
}

Props* Props::add_to_child_array(const std::string& k, const Props& c) {
    if (!child_arrays_.count(k)) child_array_keys_.push_back(k);
    child_arrays_[k].emplace_back(new Props(c));
    return this;
}

void Props::clear() {
    props_.clear(); keys_.clear();
    children_.clear(); child_keys_.clear();
    arrays_.clear(); array_keys_.clear();
    child_arrays_.clear(); child_array_keys_.clear();
}

void Props::copy_from(const Props& o) {
    for (auto& k : o.keys_) set(k, o.props_.at(k));
    for (auto& k : o.child_keys_) set_child(k, *o.children_.at(k));
    for (auto& k : o.array_keys_)
        for (auto& v : o.arrays_.at(k)) add_to_array(k, v);
    for (auto& k : o.child_array_keys_)
        for (auto& c : o.child_arrays_.at(k)) add_to_child_array(k, *c);
}

// ---------------------------------------------------------------------------
// Minimal JSON reader / writer.
// ---------------------------------------------------------------------------
namespace {

struct Value {
    enum Kind { STRING, OBJECT, ARRAY, OTHER } kind = OTHER;
    std::string str;
    std::map<std::string, Value> obj;   // sorted keys
    std::vector<Value> arr;
};

struct Reader {
    const std::string& s;
    size_t i = 0;
    explicit Reader(const std::string& s) : s(s) {}

    void ws() { while (i < s.size() && std::isspace((unsigned char)s[i])) ++i; }
    [[noreturn]] void fail(const char* what) {
        throw SgError(std::string("JSON parse error: ") + what + " at offset " + std::to_string(i));
    }
    char peek() { ws(); if (i >= s.size()) fail("unexpected end"); return s[i]; }

    std::string string() {
        if (peek() != '"') fail("expected string");
        ++i;
        std::string out;
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) fail("bad escape");
                char e = s[i++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (i + 4 > s.size()) fail("bad unicode escape");
                        unsigned cp = std::strtoul(s.substr(i, 4).c_str(), nullptr, 16);
                        i += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F));
                               out += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i >= s.size()) fail("unterminated string");
        ++i;
        return out;
    }

    Value value() {
        Value v;
        char c = peek();
        if (c == '"') { v.kind = Value::STRING; v.str = string(); }
        else if (c == '{') {
            v.kind = Value::OBJECT; ++i;
            if (peek() == '}') { ++i; return v; }
            for (;;) {
                std::string k = string();
                if (peek() != ':') fail("expected ':'");
                ++i;
                v.obj[k] = value();
                char d = peek(); ++i;
                if (d == '}') break;
                if (d != ',') fail("expected ',' or '}'");
            }
        } else if (c == '[') {
            v.kind = Value::ARRAY; ++i;
            if (peek() == ']') { ++i; return v; }
            for (;;) {
                v.arr.push_back(value());
                char d = peek(); ++i;
                if (d == ']') break;
                if (d != ',') fail("expected ',' or ']'");
            }
        } else {
            // number / true / false / null: skipped like the reference loader
            while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '-' ||
                                    s[i] == '+' || s[i] == '.'))
                ++i;
        }
        return v;
    }
};

Props to_props(const Value& o) {
    Props p;
    for (auto& kv : o.obj) {
        const Value& v = kv.second;
        if (v.kind == Value::STRING) p.set(kv.first, v.str);
        else if (v.kind == Value::OBJECT) p.set_child(kv.first, to_props(v));
        else if (v.kind == Value::ARRAY)
            for (auto& item : v.arr) {
                if (item.kind == Value::OBJECT) p.add_to_child_array(kv.first, to_props(item));
                else if (item.kind == Value::STRING) p.add_to_array(kv.first, item.str);
            }
    }
    return p;
}

void quote(std::ostringstream& os, const std::string& s) {
    os << '"';
    for (char c : s) {
        switch (c) {
            case '"': os << "\\\""; break;
            case '\\': os << "\\\\"; break;
            case '\n': os << "\\n"; break;
            case '\t': os << "\\t"; break;
            default: os << c;
        }
    }
    os << '"';
}

void write(std::ostringstream& os, const Props& p) {
    os << '{';
    bool first = true;
    auto sep = [&]() { if (!first) os << ','; first = false; };
    for (auto& k : p.keys()) {
        std::string v = p.get(k);
        if (v.empty()) continue;
        sep(); quote(os, k); os << ':'; quote(os, v);
    }
    for (auto& k : p.child_keys()) { sep(); quote(os, k); os << ':'; write(os, *p.child(k)); }
    for (auto& k : p.array_keys()) {
        auto a = p.array(k);
        if (a.empty()) continue;
        sep(); quote(os, k); os << ":[";
        for (size_t j = 0; j < a.size(); ++j) { if (j) os << ','; quote(os, a[j]); }
        os << ']';
    }
    for (auto& k : p.child_array_keys()) {
        auto a = p.child_array(k);
        if (a.empty()) continue;
        sep(); quote(os, k); os << ":[";
        for (size_t j = 0; j < a.size(); ++j) { if (j) os << ','; write(os, *a[j]); }
        os << ']';
    }
    os << '}';
}

}  // namespace

Props parse_json(const std::string& text) {
    Reader r(text);
    Value v = r.value();
    if (v.kind != Value::OBJECT) throw SgError("JSON parse error: top level must be an object");
    return to_props(v);
}

std::string write_json(const Props& p) {
    std::ostringstream os;
    write(os, p);
    return os.str();
}

}  // namespace sg
