// sd_json.h -- a small JSON reader for the scene files (objects, arrays,
// numbers, strings, booleans, null).  Written for this library; the
// reference uses the vendored nlohmann::json for the same schema
// (src/engine/engine.cpp:65-108).
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace sd {

struct JsonValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JsonValue> arr;
    std::vector<std::pair<std::string, JsonValue>> obj;  // keeps file order

    const JsonValue* get(const std::string& k) const {
        for (auto& kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string& text) : s_(text), i_(0) {}

    bool parse(JsonValue* out, std::string* err) {
        skip_ws();
        if (!value(out, 0)) {
            *err = err_.empty() ? "malformed JSON" : err_;
            return false;
        }
        skip_ws();
        if (i_ != s_.size()) {
            *err = "trailing characters after JSON value at offset " + std::to_string(i_);
            return false;
        }
        return true;
    }

  private:
    const std::string& s_;
    size_t i_;
    std::string err_;

    void skip_ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) ++i_;
    }
    bool fail(const char* what) {
        if (err_.empty()) err_ = std::string(what) + " at offset " + std::to_string(i_);
        return false;
    }
    bool literal(const char* lit) {
        size_t n = 0;
        while (lit[n]) ++n;
        if (s_.compare(i_, n, lit) != 0) return fail("bad literal");
        i_ += n;
        return true;
    }
    bool value(JsonValue* v, int depth) {
        if (depth > 64) return fail("nesting too deep");
        skip_ws();
        if (i_ >= s_.size()) return fail("unexpected end");
        char c = s_[i_];
        if (c == '{') return object(v, depth);
        if (c == '[') return array(v, depth);
        if (c == '"') {
            v->kind = JsonValue::String;
            return string(&v->str);
        }
        if (c == 't') {
            v->kind = JsonValue::Bool;
            v->b = true;
            return literal("true");
        }
        if (c == 'f') {
            v->kind = JsonValue::Bool;
            v->b = false;
            return literal("false");
        }
        if (c == 'n') {
            v->kind = JsonValue::Null;
            return literal("null");
        }
        return number(v);
    }
    bool number(JsonValue* v) {
        const char* begin = s_.c_str() + i_;
        char* end = nullptr;
        double d = std::strtod(begin, &end);
        if (end == begin) return fail("expected a value");
        i_ += (size_t)(end - begin);
        v->kind = JsonValue::Number;
        v->num = d;
        return true;
    }
    bool string(std::string* out) {
        ++i_;  // opening quote
        out->clear();
        while (i_ < s_.size()) {
            char c = s_[i_++];
            if (c == '"') return true;
            if (c == '\\') {
                if (i_ >= s_.size()) break;
                char e = s_[i_++];
                switch (e) {
                    case '"': out->push_back('"'); break;
                    case '\\': out->push_back('\\'); break;
                    case '/': out->push_back('/'); break;
                    case 'b': out->push_back('\b'); break;
                    case 'f': out->push_back('\f'); break;
                    case 'n': out->push_back('\n'); break;
                    case 'r': out->push_back('\r'); break;
                    case 't': out->push_back('\t'); break;
                    case 'u':
                        if (i_ + 4 > s_.size()) return fail("bad \\u escape");
                        out->push_back('?');  // scene files carry no non-ASCII names
                        i_ += 4;
                        break;
                    default: return fail("bad escape");
                }
            } else {
                out->push_back(c);
            }
        }
        return fail("unterminated string");
    }
    bool array(JsonValue* v, int depth) {
        v->kind = JsonValue::Array;
        ++i_;
        skip_ws();
        if (i_ < s_.size() && s_[i_] == ']') {
            ++i_;
            return true;
        }
        while (true) {
            JsonValue e;
            if (!value(&e, depth + 1)) return false;
            v->arr.push_back(std::move(e));
            skip_ws();
            if (i_ < s_.size() && s_[i_] == ',') {
                ++i_;
                continue;
            }
            if (i_ < s_.size() && s_[i_] == ']') {
                ++i_;
                return true;
            }
            return fail("expected , or ]");
        }
    }
    bool object(JsonValue* v, int depth) {
        v->kind = JsonValue::Object;
        ++i_;
        skip_ws();
        if (i_ < s_.size() && s_[i_] == '}') {
            ++i_;
            return true;
        }
        while (true) {
            skip_ws();
            if (i_ >= s_.size() || s_[i_] != '"') return fail("expected key");
            std::string k;
            if (!string(&k)) return false;
            skip_ws();
            if (i_ >= s_.size() || s_[i_] != ':') return fail("expected :");
            ++i_;
            JsonValue e;
            if (!value(&e, depth + 1)) return false;
            v->obj.emplace_back(std::move(k), std::move(e));
            skip_ws();
            if (i_ < s_.size() && s_[i_] == ',') {
                ++i_;
                continue;
            }
            if (i_ < s_.size() && s_[i_] == '}') {
                ++i_;
                return true;
            }
            return fail("expected , or }");
        }
    }
};

}  // namespace sd
