// json_lite.h -- minimal JSON reader for ld-decode sidecars (objects, arrays,
// strings, numbers, booleans, null). Numbers are kept as double plus the
// integer value when exact.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace chdg::json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::map<std::string, Value> obj;

    const Value *get(const std::string &key) const
    {
        if (kind != Object) return nullptr;
        auto it = obj.find(key);
        return it == obj.end() ? nullptr : &it->second;
    }
    bool is_number() const { return kind == Number; }
};

// Parses text; on error returns false and fills err with "offset N: reason".
bool parse(const std::string &text, Value &out, std::string &err);

}  // namespace chdg::json
