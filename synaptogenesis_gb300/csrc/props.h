// String-keyed property tree used by every configuration object.
//
// Mirrors the reference's PropertyConfig (src/core/util/property_config.h:26-114):
// scalar properties are strings kept in insertion order, plus ordered children,
// string arrays and child arrays.  Typed getters follow std::stoi / std::stof /
// "== true" semantics (property_config.cpp:94-119).
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sg {

struct SgError : std::runtime_error {
    explicit SgError(const std::string& m) : std::runtime_error(m) {}
};

class Props {
  public:
    Props() = default;
    Props(const Props& o) { copy_from(o); }
    Props& operator=(const Props& o) {
        if (this != &o) { clear(); copy_from(o); }
        return *this;
    }

    bool has(const std::string& k) const { return props_.count(k) > 0; }
    std::string get(const std::string& k, const std::string& def = "") const {
        auto it = props_.find(k);
        return it == props_.end() ? def : it->second;
    }
    const char* get_c_str(const std::string& k) const {
        auto it = props_.find(k);
        return it == props_.end() ? nullptr : it->second.c_str();
    }
    int get_int(const std::string& k, int def) const;
    float get_float(const std::string& k, float def) const;
    bool get_bool(const std::string& k, bool def) const {
        return has(k) ? get(k) == "true" : def;
    }
    Props* set(const std::string& k, const std::string& v);

    bool has_child(const std::string& k) const { return children_.count(k) > 0; }
    Props* child(const std::string& k) const {
        auto it = children_.find(k);
        return it == children_.end() ? nullptr : it->second.get();
    }
    Props* set_child(const std::string& k, const Props& c);

    bool has_array(const std::string& k) const { return arrays_.count(k) > 0; }
    std::vector<std::string> array(const std::string& k) const {
        auto it = arrays_.find(k);
        return it == arrays_.end() ? std::vector<std::string>() : it->second;
    }
    Props* add_to_array(const std::string& k, const std::string& v);

    bool has_child_array(const std::string& k) const { return child_arrays_.count(k) > 0; }
    std::vector<Props*> child_array(const std::string& k) const;
    Props* add_to_child_array(const std::string& k, const Props& c);

    const std::vector<std::string>& keys() const { return keys_; }
    const std::vector<std::string>& child_keys() const { return child_keys_; }
    const std::vector<std::string>& array_keys() const { return array_keys_; }
    const std::vector<std::string>& child_array_keys() const { return child_array_keys_; }

  private:
    void clear();
    void copy_from(const Props& o);

    std::map<std::string, std::string> props_;
    std::vector<std::string> keys_;
    std::map<std::string, std::unique_ptr<Props>> children_;
    std::vector<std::string> child_keys_;
    std::map<std::string, std::vector<std::string>> arrays_;
    std::vector<std::string> array_keys_;
    std::map<std::string, std::vector<std::unique_ptr<Props>>> child_arrays_;
    std::vector<std::string> child_array_keys_;
};

// JSON <-> Props.  Only string values, objects and arrays are kept; numbers,
// booleans and null are ignored, as in the reference loader
// (src/core/builder.cpp:15-39).  Object keys come out in sorted order, as the
// reference's JSON library stores them in an ordered map.
Props parse_json(const std::string& text);
std::string write_json(const Props& p);

}  // namespace sg
