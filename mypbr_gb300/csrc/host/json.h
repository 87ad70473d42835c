// A small JSON reader (RFC 8259) for glTF documents: the whole text into a
// tree of values. Numbers are doubles, strings UTF-8 (\u escapes decoded,
// surrogate pairs joined); object keys keep their order.
#pragma once

#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace mypbr_host {

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool boolean = false;
    double number = 0;
    std::string text;
    std::vector<Json> items;                         // Array
    std::vector<std::pair<std::string, Json>> members;  // Object

    // Member of an object, or nullptr (also when this is not an object).
    const Json* find(const std::string& key) const;
    // Element of an array, or nullptr.
    const Json* at(size_t k) const { return kind == Array && k < items.size() ? &items[k] : nullptr; }
    size_t size() const { return kind == Array ? items.size() : 0; }

    // Typed reads of members with defaults.
    double num(const std::string& key, double fallback) const;
    long long integer(const std::string& key, long long fallback) const;
    std::string str(const std::string& key, const std::string& fallback = "") const;
    bool flag(const std::string& key, bool fallback) const;
};

// Parses text; false with a message (and the byte offset) if it is not JSON.
bool parse_json(const char* text, size_t size, Json& out, std::string& error);

}  // namespace mypbr_host
