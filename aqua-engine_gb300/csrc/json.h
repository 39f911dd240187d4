// json.h — a small JSON reader for the scene and integrator files
// (scenes/cbox.json, scenes/room.json, scenes/integrator.json). The reference
// reads them with serde_json (Cargo.toml:15-16); this is a standalone
// recursive-descent parser (RFC 8259) that reports the byte offset of the
// first error.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace aq {

struct JsonError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;  // insertion order kept

    bool is_object() const { return kind == Object; }
    bool is_array() const { return kind == Array; }
    bool is_number() const { return kind == Number; }
    bool is_string() const { return kind == String; }
    const Json* find(const std::string& key) const {
        for (auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    const Json& at(const std::string& key) const {
        const Json* j = find(key);
        if (!j) throw JsonError("missing key \"" + key + "\"");
        return *j;
    }
    double as_number() const {
        if (kind != Number) throw JsonError("expected a number");
        return num;
    }
    const std::string& as_string() const {
        if (kind != String) throw JsonError("expected a string");
        return str;
    }
};

Json json_parse(const std::string& text);  // throws JsonError

}  // namespace aq
