// json.hpp -- minimal JSON reader for the engine config (objects, arrays, strings,
// numbers, booleans, null).  Numbers keep their source text so integers parse exactly.
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace epi {
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    std::string text;  // number text or string contents
    std::vector<Value> items;
    std::vector<std::pair<std::string, Value>> members;

    const Value* get(const std::string& key) const {
        if (kind != Object) return nullptr;
        for (const auto& m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
    double as_double() const {
        if (kind != Number) throw std::runtime_error("expected a number");
        return std::strtod(text.c_str(), nullptr);
    }
    // Unsigned integer that must be written as an integer literal (serde rejects 1.5 for u32).
    unsigned long long as_uint() const {
        if (kind != Number) throw std::runtime_error("expected an integer");
        if (text.find_first_of(".eE-") != std::string::npos) throw std::runtime_error("expected a non-negative integer, got " + text);
        return std::strtoull(text.c_str(), nullptr, 10);
    }
};

class Parser {
  public:
    explicit Parser(const std::string& s) : s_(s) {}
    Value parse() {
        Value v = value();
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return v;
    }

  private:
    const std::string& s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const std::string& what) {
        throw std::runtime_error("JSON parse error at offset " + std::to_string(i_) + ": " + what);
    }
    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\r' || s_[i_] == '\t')) ++i_;
    }
    bool eat(char c) {
        ws();
        if (i_ < s_.size() && s_[i_] == c) { ++i_; return true; }
        return false;
    }
    void expect(char c) {
        if (!eat(c)) fail(std::string("expected '") + c + "'");
    }
    Value value() {
        ws();
        if (i_ >= s_.size()) fail("unexpected end");
        char c = s_[i_];
        if (c == '{') return object();
        if (c == '[') return array();
        if (c == '"') { Value v; v.kind = Value::String; v.text = str(); return v; }
        if (s_.compare(i_, 4, "true") == 0) { i_ += 4; Value v; v.kind = Value::Bool; v.b = true; return v; }
        if (s_.compare(i_, 5, "false") == 0) { i_ += 5; Value v; v.kind = Value::Bool; return v; }
        if (s_.compare(i_, 4, "null") == 0) { i_ += 4; return Value(); }
        if (c == '-' || (c >= '0' && c <= '9')) return number();
        fail("unexpected character");
    }
    Value number() {
        size_t start = i_;
        if (s_[i_] == '-') ++i_;
        while (i_ < s_.size() && (isdigit((unsigned char)s_[i_]) || s_[i_] == '.' || s_[i_] == 'e' || s_[i_] == 'E' ||
                                  s_[i_] == '+' || s_[i_] == '-'))
            ++i_;
        Value v;
        v.kind = Value::Number;
        v.text = s_.substr(start, i_ - start);
        char* end = nullptr;
        std::strtod(v.text.c_str(), &end);
        if (end != v.text.c_str() + v.text.size()) fail("bad number " + v.text);
        return v;
    }
    std::string str() {
        expect('"');
        std::string out;
        while (true) {
            if (i_ >= s_.size()) fail("unterminated string");
            char c = s_[i_++];
            if (c == '"') break;
            if (c == '\\') {
                if (i_ >= s_.size()) fail("bad escape");
                char e = s_[i_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (i_ + 4 > s_.size()) fail("bad \\u escape");
                        unsigned cp = (unsigned)std::strtoul(s_.substr(i_, 4).c_str(), nullptr, 16);
                        i_ += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: out += e; break;
                }
            } else {
                out += c;
            }
        }
        return out;
    }
    Value array() {
        expect('[');
        Value v;
        v.kind = Value::Array;
        if (eat(']')) return v;
        do { v.items.push_back(value()); } while (eat(','));
        expect(']');
        return v;
    }
    Value object() {
        expect('{');
        Value v;
        v.kind = Value::Object;
        if (eat('}')) return v;
        do {
            ws();
            std::string k = str();
            expect(':');
            v.members.emplace_back(k, value());
        } while (eat(','));
        expect('}');
        return v;
    }
};

inline Value parse(const std::string& s) { return Parser(s).parse(); }

}  // namespace json
}  // namespace epi
