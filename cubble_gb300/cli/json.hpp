// Minimal JSON reader for the simulation input (input_parameters.json):
// objects, arrays, numbers, strings, true/false/null. Numbers are doubles
// (the input writes counts as 1e5). Parse errors throw std::runtime_error
// with the byte offset.
#pragma once

#include <cctype>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cbj {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::map<std::string, Value> obj;

    bool has(const std::string &key) const { return kind == Object && obj.count(key) > 0; }
    const Value &operator[](const std::string &key) const {
        if (kind != Object) throw std::runtime_error("json: '" + key + "' looked up in a non-object");
        auto it = obj.find(key);
        if (it == obj.end()) throw std::runtime_error("json: missing key '" + key + "'");
        return it->second;
    }
    Value &at_path(const std::vector<std::string> &path) {
        Value *v = this;
        for (const std::string &k : path) {
            if (v->kind != Object) throw std::runtime_error("json: '" + k + "' looked up in a non-object");
            auto it = v->obj.find(k);
            if (it == v->obj.end()) throw std::runtime_error("json: missing key '" + k + "'");
            v = &it->second;
        }
        return *v;
    }
    double number() const {
        if (kind == Number) return num;
        if (kind == Bool) return b ? 1.0 : 0.0;
        throw std::runtime_error("json: value is not a number");
    }
    int integer() const { return (int)number(); }
    const std::string &string() const {
        if (kind != String) throw std::runtime_error("json: value is not a string");
        return str;
    }
};

class Parser {
  public:
    explicit Parser(const std::string &text) : s_(text) {}
    Value parse() {
        Value v = value();
        ws();
        if (p_ != s_.size()) fail("trailing characters");
        return v;
    }

  private:
    const std::string &s_;
    size_t p_ = 0;

    [[noreturn]] void fail(const char *what) const {
        throw std::runtime_error(std::string("json: ") + what + " at byte " + std::to_string(p_));
    }
    void ws() {
        while (p_ < s_.size() && std::isspace((unsigned char)s_[p_])) p_++;
    }
    bool eat(char ch) {
        ws();
        if (p_ < s_.size() && s_[p_] == ch) {
            p_++;
            return true;
        }
        return false;
    }
    void expect(char ch) {
        if (!eat(ch)) fail("unexpected character");
    }
    Value value() {
        ws();
        if (p_ >= s_.size()) fail("unexpected end");
        const char ch = s_[p_];
        Value v;
        if (ch == '{') {
            p_++;
            v.kind = Value::Object;
            if (eat('}')) return v;
            do {
                ws();
                std::string key = string_literal();
                expect(':');
                v.obj[key] = value();
            } while (eat(','));
            expect('}');
        } else if (ch == '[') {
            p_++;
            v.kind = Value::Array;
            if (eat(']')) return v;
            do {
                v.arr.push_back(value());
            } while (eat(','));
            expect(']');
        } else if (ch == '"') {
            v.kind = Value::String;
            v.str = string_literal();
        } else if (s_.compare(p_, 4, "true") == 0) {
            p_ += 4;
            v.kind = Value::Bool;
            v.b = true;
        } else if (s_.compare(p_, 5, "false") == 0) {
            p_ += 5;
            v.kind = Value::Bool;
        } else if (s_.compare(p_, 4, "null") == 0) {
            p_ += 4;
        } else {
            const char *begin = s_.c_str() + p_;
            char *end = nullptr;
            v.num = std::strtod(begin, &end);
            if (end == begin) fail("bad value");
            p_ += (size_t)(end - begin);
            v.kind = Value::Number;
        }
        return v;
    }
    std::string string_literal() {
        if (p_ >= s_.size() || s_[p_] != '"') fail("expected a string");
        p_++;
        std::string out;
        while (p_ < s_.size() && s_[p_] != '"') {
            char ch = s_[p_++];
            if (ch == '\\') {
                if (p_ >= s_.size()) fail("bad escape");
                const char e = s_[p_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (p_ + 4 > s_.size()) fail("bad escape");
                        const unsigned cp = (unsigned)std::stoul(s_.substr(p_, 4), nullptr, 16);
                        p_ += 4;
                        out += cp < 0x80 ? (char)cp : '?';
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += ch;
            }
        }
        if (p_ >= s_.size()) fail("unterminated string");
        p_++;
        return out;
    }
};

inline Value parse(const std::string &text) { return Parser(text).parse(); }

}  // namespace cbj
