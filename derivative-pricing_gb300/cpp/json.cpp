// json.cpp -- parser and writer for the CLI's flat JSON objects (json.hpp).
#include "json.hpp"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <string>

namespace mcdjson {

namespace {

class Reader {
  public:
    explicit Reader(std::string_view t) : t_(t) {}

    Object top_level() {
        ws();
        expect('{');
        Object obj;
        ws();
        if (peek() == '}') {
            ++i_;
        } else {
            for (;;) {
                ws();
                std::string key = string();
                ws();
                expect(':');
                ws();
                obj.emplace_back(std::move(key), value(true));
                ws();
                if (peek() == ',') {
                    ++i_;
                    continue;
                }
                expect('}');
                break;
            }
        }
        ws();
        if (i_ != t_.size()) fail("trailing characters after the object");
        return obj;
    }

  private:
    std::string_view t_;
    size_t i_ = 0;

    [[noreturn]] void fail(const std::string& what) const {
        throw ParseError("invalid JSON at offset " + std::to_string(i_) + ": " + what);
    }
    char peek() const { return i_ < t_.size() ? t_[i_] : '\0'; }
    void ws() {
        while (i_ < t_.size() && std::isspace(static_cast<unsigned char>(t_[i_]))) ++i_;
    }
    void expect(char c) {
        if (peek() != c) fail(std::string("expected '") + c + "'");
        ++i_;
    }
    bool literal(std::string_view word) {
        if (t_.substr(i_, word.size()) == word) {
            i_ += word.size();
            return true;
        }
        return false;
    }

    std::string string() {
        expect('"');
        std::string out;
        while (i_ < t_.size() && t_[i_] != '"') {
            char c = t_[i_++];
            if (c == '\\') {
                if (i_ >= t_.size()) fail("unterminated escape");
                const char e = t_[i_++];
                switch (e) {
                    case '"': out += '"'; break;
                    case '\\': out += '\\'; break;
                    case '/': out += '/'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'n': out += '\n'; break;
                    case 'r': out += '\r'; break;
                    case 't': out += '\t'; break;
                    case 'u': {
                        if (i_ + 4 > t_.size()) fail("short \\u escape");
                        const unsigned cp = static_cast<unsigned>(std::strtoul(std::string(t_.substr(i_, 4)).c_str(), nullptr, 16));
                        i_ += 4;
                        if (cp < 0x80) {
                            out += static_cast<char>(cp);
                        } else if (cp < 0x800) {
                            out += static_cast<char>(0xC0 | (cp >> 6));
                            out += static_cast<char>(0x80 | (cp & 0x3F));
                        } else {
                            out += static_cast<char>(0xE0 | (cp >> 12));
                            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
                            out += static_cast<char>(0x80 | (cp & 0x3F));
                        }
                        break;
                    }
                    default: fail("unknown escape");
                }
            } else {
                out += c;
            }
        }
        expect('"');
        return out;
    }

    double number() {
        const size_t start = i_;
        if (peek() == '-' || peek() == '+') ++i_;
        while (i_ < t_.size() && (std::isdigit(static_cast<unsigned char>(t_[i_])) || t_[i_] == '.' || t_[i_] == 'e' ||
                                  t_[i_] == 'E' || t_[i_] == '-' || t_[i_] == '+'))
            ++i_;
        const std::string s(t_.substr(start, i_ - start));
        char* end = nullptr;
        const double v = std::strtod(s.c_str(), &end);
        if (s.empty() || end != s.c_str() + s.size()) fail("bad number");
        return v;
    }

    Value value(bool allow_array) {
        const char c = peek();
        if (c == '"') return Value::string(string());
        if (literal("true")) return Value::boolean(true);
        if (literal("false")) return Value::boolean(false);
        if (literal("null")) return Value::null();
        if (c == '[' && allow_array) {
            ++i_;
            std::vector<Value> items;
            ws();
            if (peek() == ']') {
                ++i_;
                return Value::array(std::move(items));
            }
            for (;;) {
                ws();
                items.push_back(value(false));
                ws();
                if (peek() == ',') {
                    ++i_;
                    continue;
                }
                expect(']');
                break;
            }
            return Value::array(std::move(items));
        }
        if (c == '-' || c == '+' || std::isdigit(static_cast<unsigned char>(c))) return Value::number(number());
        fail("unsupported value (only null, bool, number, string and flat arrays)");
    }
};

void escaped(std::string& out, const std::string& s) {
    out += '"';
    for (char c : s) {
        switch (c) {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\n': out += "\\n"; break;
            case '\t': out += "\\t"; break;
            case '\r': out += "\\r"; break;
            default: out += c;
        }
    }
    out += '"';
}

void write(std::string& out, const Value& v, int digits) {
    switch (v.type) {
        case Value::Type::Null: out += "null"; break;
        case Value::Type::Bool: out += v.b ? "true" : "false"; break;
        case Value::Type::Number: {
            char buf[64];
            const int n = std::snprintf(buf, sizeof buf, "%.*g", digits, v.num);
            out.append(buf, static_cast<size_t>(n));
            break;
        }
        case Value::Type::String: escaped(out, v.str); break;
        case Value::Type::Array: {
            out += '[';
            for (size_t i = 0; i < v.items.size(); ++i) {
                if (i) out += ',';
                write(out, v.items[i], digits);
            }
            out += ']';
            break;
        }
    }
}

}  // namespace

Object parse_object(std::string_view text) { return Reader(text).top_level(); }

std::string serialize(const Object& obj, int digits) {
    std::string out = "{";
    for (size_t i = 0; i < obj.size(); ++i) {
        if (i) out += ',';
        escaped(out, obj[i].first);
        out += ':';
        write(out, obj[i].second, digits);
    }
    out += '}';
    return out;
}

const Value* find(const Object& obj, std::string_view key) {
    for (const auto& kv : obj)
        if (kv.first == key) return &kv.second;
    return nullptr;
}

}  // namespace mcdjson
