// json.hpp -- the JSON subset of the CLI schema: one flat object of null,
// bool, number, string and (for the batch request only) arrays of numbers or
// strings.  Numbers are written with "%.10g" by default and objects keep
// insertion order, as the reference CLI prints them (src/core/json.cpp:276-321);
// 17 digits round-trip a double exactly.
#pragma once

#include <stdexcept>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

namespace mcdjson {

struct Value {
    enum class Type { Null, Bool, Number, String, Array };
    Type type = Type::Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> items;

    static Value null() { return Value{}; }
    static Value boolean(bool v) {
        Value x;
        x.type = Type::Bool;
        x.b = v;
        return x;
    }
    static Value number(double v) {
        Value x;
        x.type = Type::Number;
        x.num = v;
        return x;
    }
    static Value string(std::string v) {
        Value x;
        x.type = Type::String;
        x.str = std::move(v);
        return x;
    }
    static Value array(std::vector<Value> v) {
        Value x;
        x.type = Type::Array;
        x.items = std::move(v);
        return x;
    }
};

using Object = std::vector<std::pair<std::string, Value>>;

struct ParseError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

Object parse_object(std::string_view text);
std::string serialize(const Object& obj, int digits = 10);
const Value* find(const Object& obj, std::string_view key);

}  // namespace mcdjson
